/*
 * devmem.cu -- the library's device memory: one stream-ordered pool per GPU.
 *
 * Every device buffer the library owns (resident graphs, traversal
 * workspaces, ingest and batch scratch, server pools) comes from
 * tbfs::dev_alloc and goes back through tbfs::dev_free.  The pool keeps
 * freed memory mapped up to a threshold, so a graph that is built, queried
 * and destroyed again and again (a host-buffer caller of the reference's
 * entry points does exactly that on every call) reuses its memory instead of
 * mapping and unmapping hundreds of MB each time.
 *
 * Semantics match cudaMalloc / cudaFree as the library used them:
 *   dev_alloc  returns memory that every stream may use as soon as it
 *              returns (the allocation is made on the pool's own stream,
 *              which is then synchronised);
 *   dev_free   waits for all work on the device first, as cudaFree does,
 *              then returns the block to the pool.
 *
 * Environment:
 *   TBFS_POOL_KEEP_MB   memory kept mapped by the pool once idle (default
 *                       8192; 0 returns everything at each synchronisation)
 *   TBFS_POOL_POISON    when set to a non-zero value, every allocation is
 *                       filled with 0xA5 bytes, so that code relying on
 *                       fresh memory reading as zero fails its tests
 */
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "tbfs_internal.h"

namespace tbfs {

namespace {

constexpr int kMaxDevices = 64;

struct DevicePool {
  std::once_flag once;
  cudaError_t init_err = cudaSuccess;
  cudaMemPool_t pool = nullptr;
  cudaStream_t stream = nullptr;
};

DevicePool g_pools[kMaxDevices];

unsigned long long keep_bytes() {
  const char *s = std::getenv("TBFS_POOL_KEEP_MB");
  if (!s || !*s) return 8192ull << 20;
  char *end = nullptr;
  const unsigned long long mb = std::strtoull(s, &end, 10);
  return mb << 20;
}

bool poison() {
  const char *s = std::getenv("TBFS_POOL_POISON");
  return s && *s && *s != '0';
}

void init_pool(DevicePool &dp, int dev) {
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaError_t e = cudaMemPoolCreate(&dp.pool, &props);
  if (e == cudaSuccess) {
    unsigned long long keep = keep_bytes(); /* the attribute is a 64-bit value */
    e = cudaMemPoolSetAttribute(dp.pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&dp.stream, cudaStreamNonBlocking);
  dp.init_err = e;
}

cudaError_t pool_of(int dev, DevicePool **out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  DevicePool &dp = g_pools[dev];
  std::call_once(dp.once, init_pool, std::ref(dp), dev);
  *out = &dp;
  return dp.init_err;
}

}  // namespace

cudaError_t dev_alloc(void **p, size_t bytes) {
  *p = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  DevicePool *dp = nullptr;
  if (e == cudaSuccess) e = pool_of(dev, &dp);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, dp->pool, dp->stream);
  if (e == cudaSuccess && poison()) e = cudaMemsetAsync(*p, 0xA5, bytes, dp->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(dp->stream);
  if (e != cudaSuccess) {
    if (*p && dp) cudaFreeAsync(*p, dp->stream);
    *p = nullptr;
  }
  return e;
}

cudaError_t dev_free(void *p) {
  if (!p) return cudaSuccess;
  cudaPointerAttributes at = {};
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) return e;
  int cur = 0;
  e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return e;
  if (at.device != cur) cudaSetDevice(at.device);
  DevicePool *dp = nullptr;
  e = pool_of(at.device, &dp);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaFreeAsync(p, dp->stream);
  if (at.device != cur) cudaSetDevice(cur);
  return e;
}

cudaError_t dev_trim(size_t keep) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  DevicePool *dp = nullptr;
  if (e == cudaSuccess) e = pool_of(dev, &dp);
  if (e == cudaSuccess) e = cudaStreamSynchronize(dp->stream);
  if (e == cudaSuccess) e = cudaMemPoolTrimTo(dp->pool, keep);
  return e;
}

}  // namespace tbfs

extern "C" tbfs_status tbfs_release_cached_memory(void) {
  const cudaError_t e = tbfs::dev_trim(0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    tbfs_set_error("tbfs_release_cached_memory: %s", cudaGetErrorString(e));
    return TBFS_ERR_CUDA;
  }
  return TBFS_OK;
}
