/*
 * noalloc.cu -- tbfs_bfs_noalloc: one BFS that allocates nothing.
 *
 * Who needs it: callers that cannot let a library call cudaMalloc/cudaFree
 * -- a host framework that hands out all device memory from its own pool
 * (a database or serving engine with an arena allocator, where an
 * allocation behind its back fails or breaks its memory accounting), and
 * latency-critical loops that must not take the device-wide
 * synchronisation cudaMalloc/cudaFree may impose.  Such a caller passes the
 * graph and the outputs as device pointers; the frontier queues and the
 * control block the traversal needs live in one file-scope device array,
 * g_noalloc_scratch, sized for graphs of up to TBFS_NOALLOC_MAX_VERTICES
 * vertices.  That array is part of the library's device code: once that code
 * is loaded on a GPU, the GPU holds the array (about 36 MB) until the process
 * exits.
 *
 * Host code cannot use the array's name as a device address; on the first
 * call on each device (with that device current) the address is looked up
 * with cudaGetSymbolAddress and cached for the device's current context.
 * CUDA loads device code lazily, so when nothing else of the library ran on
 * that device yet, this first call is also the moment the 36 MB are
 * committed: make it as a warm-up before the host framework reserves the
 * device memory it manages, and before any stream capture.  If the memory
 * is not there, the call fails with TBFS_ERR_OUT_OF_MEMORY.  A new context
 * on the device (after cudaDeviceReset) gets a fresh lookup.  Every call
 * waits for its traversal to finish on the caller's stream.  Every call
 * shares the one array: the control block is cleared at the start of each
 * call, and two calls whose work overlaps on the GPU (different streams or
 * host threads without ordering) race on it.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "tbfs.h"
#include "tbfs_internal.h"

namespace {

constexpr size_t kCtlBytes = 8192; /* control block + validation flag */
constexpr size_t kQueueBytes = (size_t)TBFS_NOALLOC_MAX_VERTICES * sizeof(int);
constexpr size_t kBitmapBytes = (size_t)TBFS_NOALLOC_MAX_VERTICES / 8;
constexpr size_t kScratchBytes = kCtlBytes + 9 * kQueueBytes + 4 * kBitmapBytes;
constexpr size_t kFlagOffset = kCtlBytes - 256;
static_assert(sizeof(tbfs::BfsCtl) <= kFlagOffset, "control block must fit its slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
  bool ready = false;
  unsigned long long ctx_id = 0;    /* context the address belongs to */
  unsigned char *scratch = nullptr; /* device address of g_noalloc_scratch */
  tbfs::LaunchGeom geom;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

tbfs_status fail(tbfs_status s, const char *msg) {
  tbfs_set_error("%s", msg);
  return s;
}

tbfs_status cuda_fail(cudaError_t e, const char *what) {
  tbfs_set_error("tbfs_bfs_noalloc: %s: %s", what, cudaGetErrorString(e));
  return TBFS_ERR_CUDA;
}

/* identifier of the calling thread's current context (driver entry points
 * fetched through the runtime, so the library needs no libcuda at link time);
 * 0 if unavailable */
unsigned long long current_context_id() {
  static CUresult (*get_current)(CUcontext *) = nullptr;
  static CUresult (*get_id)(CUcontext, unsigned long long *) = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CUresult (*)(CUcontext *)>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CUresult (*)(CUcontext, unsigned long long *)>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx &&
      get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

/* once per device and context, with that device current */
tbfs_status setup_device(int dev, DeviceSetup **out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(TBFS_ERR_UNSUPPORTED, "device index too large");
  /* 0 when this thread has no current context yet: the lookup below makes
   * the device's primary context current */
  unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup &s = g_setup[dev];
  if (!s.ready || ctx == 0 || s.ctx_id != ctx) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e == cudaErrorMemoryAllocation)
      return fail(TBFS_ERR_OUT_OF_MEMORY,
                  "tbfs_bfs_noalloc: loading the library's device code (with its 36 MB scratch "
                  "array) on this device failed for lack of memory; make the first call before "
                  "device memory is reserved by the host framework");
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    e = tbfs::bfs_geometry(dev, &s.geom);
    if (e != cudaSuccess) return cuda_fail(e, "launch geometry");
    s.scratch = static_cast<unsigned char *>(ptr);
    s.ctx_id = current_context_id();
    s.ready = true;
  }
  *out = &s;
  return TBFS_OK;
}

}  // namespace

extern "C" tbfs_status tbfs_bfs_noalloc(const int32_t *d_col_ptr, const int32_t *d_row_idx,
                                        const int32_t *d_out_ptr, const int32_t *d_out_idx,
                                        int32_t n, int64_t nnz, int32_t root, int32_t mode,
                                        int32_t *d_S, int64_t *d_sigma, void *stream,
                                        tbfs_stats *stats) {
  if (n < 1 || nnz < 0 || nnz > INT32_MAX || !d_col_ptr || (nnz > 0 && !d_row_idx) || !d_S)
    return fail(TBFS_ERR_INVALID_ARG, "tbfs_bfs_noalloc: need n >= 1, 0 <= nnz <= INT32_MAX, "
                                      "col_ptr, row_idx and S");
  if (n > TBFS_NOALLOC_MAX_VERTICES)
    return fail(TBFS_ERR_UNSUPPORTED,
                "tbfs_bfs_noalloc: n exceeds TBFS_NOALLOC_MAX_VERTICES (1048576); use "
                "tbfs_graph_create_csc + tbfs_bfs for larger graphs");
  if (root < 0 || root >= n) return fail(TBFS_ERR_INVALID_ARG, "tbfs_bfs_noalloc: root outside [0, n)");
  if (mode < TBFS_MODE_AUTO || mode > TBFS_MODE_BOTTOM_UP)
    return fail(TBFS_ERR_INVALID_ARG, "tbfs_bfs_noalloc: bad mode");
  if ((d_out_ptr == nullptr && d_out_idx != nullptr) ||
      (d_out_ptr != nullptr && d_out_idx == nullptr && nnz > 0))
    return fail(TBFS_ERR_INVALID_ARG, "tbfs_bfs_noalloc: pass both out-list arrays or neither");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  DeviceSetup *ds = nullptr;
  tbfs_status st = setup_device(dev, &ds);
  if (st != TBFS_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char *base = ds->scratch;
  tbfs::BfsCtl *ctl = reinterpret_cast<tbfs::BfsCtl *>(base);
  int *flag = reinterpret_cast<int *>(base + kFlagOffset);
  int *q = reinterpret_cast<int *>(base + kCtlBytes);

  /* the array keeps the previous call's contents: clear control block + flag */
  if ((e = cudaMemsetAsync(base, 0, kCtlBytes, s)) != cudaSuccess) return cuda_fail(e, "clear");
  const bool symmetric = d_out_ptr == nullptr;
  const int32_t *rp = symmetric ? d_col_ptr : d_out_ptr;
  const int32_t *jr = symmetric ? d_row_idx : d_out_idx;
  if ((e = tbfs::validate_csc(d_col_ptr, d_row_idx, n, nnz, flag, s)) != cudaSuccess)
    return cuda_fail(e, "validate in-lists");
  if (!symmetric && (e = tbfs::validate_csc(rp, jr, n, nnz, flag, s)) != cudaSuccess)
    return cuda_fail(e, "validate out-lists");
  int hflag = 0;
  if ((e = cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "read validation flag");
  if (hflag) return fail(TBFS_ERR_INVALID_ARG, "tbfs_bfs_noalloc: malformed CSC input");

  tbfs::BfsParams p = {};
  p.cp = d_col_ptr;
  p.ic = d_row_idx;
  p.rp = rp;
  p.jr = jr;
  p.S = d_S;
  p.sigma = reinterpret_cast<unsigned long long *>(d_sigma);
  p.inv = nullptr; /* the caller's numbering is used as is */
  p.perm = nullptr;
  p.S_out = p.S;
  p.sigma_out = p.sigma;
  for (int b = 0; b < 3; ++b) {
    p.q[b] = q + (size_t)(0 + b) * TBFS_NOALLOC_MAX_VERTICES;
    p.e[b] = q + (size_t)(3 + b) * TBFS_NOALLOC_MAX_VERTICES;
    p.a[b] = q + (size_t)(6 + b) * TBFS_NOALLOC_MAX_VERTICES;
  }
  for (int b = 0; b < 4; ++b)
    p.fb[b] = reinterpret_cast<unsigned *>(base + kCtlBytes + 9 * kQueueBytes + b * kBitmapBytes);
  p.trace = nullptr;
  p.trace_cap = 0;
  p.ctl = ctl;
  p.out_edges_total = nnz;
  p.timeout_ns = 2000000000LL;
  p.n = n;
  p.root = root;
  p.mode = mode;
  p.symmetric = symmetric ? 1 : 0;
  p.alpha = 15.0f;
  p.beta = 18.0f;
  p.pull_ratio = 4.0f;
  p.inject_barrier_skip = 0;
  if ((e = tbfs::bfs_launch(p, ds->geom, s)) != cudaSuccess) return cuda_fail(e, "launch");
  tbfs::BfsCtl c;
  if ((e = cudaMemcpyAsync(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "read control block");
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->levels = c.levels;
    stats->td_levels = c.td_levels;
    stats->bu_levels = c.bu_levels;
    stats->sigma_overflow = c.sigma_overflow;
    stats->visited = c.visited;
    stats->edges = c.edges;
  }
  if (c.status != 0)
    return fail(TBFS_ERR_TIMEOUT, "tbfs_bfs_noalloc: grid barrier wait exceeded its budget");
  return TBFS_OK;
}
