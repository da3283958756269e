/*
 * cooc_engine.cu -- top-down BFS with path counts straight over a COOC
 * adjacency (entry k is the edge I[k] -> J[k]), for the drop-in COOC entry
 * point, which uploads the caller's pairs at every call.
 *
 * The reference's COOC driver (TurboBFS_COOC_TD/bfsgputdcooc_sc.cu:152-188)
 * launches, per level, an edge-parallel kernel over all nnz pairs (sigma
 * pushed from frontier sources) and a vertex kernel, with a host round trip
 * in between.  Here one persistent cooperative launch runs the levels: per
 * level every thread streams its share of the pairs (16-byte loads of four
 * sources and four destinations), tests the source against the frontier
 * bitmap of F_d, and for a frontier source claims the destination with
 * atomicCAS(S, -1, d+1) (its return value tells a new vertex from one
 * already at depth d+1) and adds sigma[src] to it.  A level costs one pass
 * over the pairs (8 bytes each) whatever the frontier's size, so the launch
 * gives up after max_levels levels (ctl->unfinished): the caller then sorts
 * the pairs into CSC once and runs the frontier-proportional engine, which
 * wins on deep graphs.  On shallow ones the pass count is small and the
 * sort (the larger part of a COOC call) is skipped.
 *
 * Bitmaps: F_d in fb[d % 3] is read, F_{d+1} in fb[(d+1) % 3] written, and
 * fb[(d+2) % 3] (F_{d-1}) cleared for F_{d+2}; the next level's size is
 * counted in cnt[(d+1) % 3].  Memory model as in the single-source engine:
 * depths and counts read with plain loads were written before the last grid
 * barrier; a depth claimed during this level is only acted on through the
 * CAS's return value.  Path counts are exact uint64; a sum reaching 2^63
 * sets ctl->sigma_overflow.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

using dev::FULL;
using dev::add_chk;
using dev::grid_barrier;
constexpr int kBlock = 256;

__device__ __forceinline__ void cooc_pair(const CoocParams &p, int d, int src, int dst,
                                          const unsigned *cur, unsigned *nxt, unsigned &taken,
                                          bool &ovf) {
  if (!((cur[(unsigned)src >> 5] >> ((unsigned)src & 31u)) & 1u)) return;
  int s = p.S[dst];
  if (s == -1) {
    s = atomicCAS(p.S + dst, -1, d + 1);
    if (s == -1) {
      atomicOr(nxt + ((unsigned)dst >> 5), 1u << ((unsigned)dst & 31u));
      ++taken;
      s = d + 1;
    }
  }
  if (s == d + 1 && p.sigma) {
    const unsigned long long x = p.sigma[src];
    add_chk(atomicAdd(p.sigma + dst, x), x, ovf);
  }
}

__global__ void __launch_bounds__(kBlock) cooc_bfs_kernel(const CoocParams p) {
  const unsigned long long gtid = (unsigned long long)blockIdx.x * kBlock + threadIdx.x;
  const unsigned long long nthreads = (unsigned long long)gridDim.x * kBlock;
  CoocCtl *ctl = p.ctl;
  const unsigned nwords = ((unsigned)p.n + 31u) >> 5;
  for (unsigned long long v = gtid; v < (unsigned long long)p.n; v += nthreads) {
    p.S[v] = (int)v == p.root ? 0 : -1;
    if (p.sigma) p.sigma[v] = (int)v == p.root ? 1ull : 0ull;
  }
  for (unsigned long long i = gtid; i < nwords; i += nthreads) {
    p.fb[0][i] = i == ((unsigned)p.root >> 5) ? 1u << ((unsigned)p.root & 31u) : 0u;
    p.fb[1][i] = 0u;
    p.fb[2][i] = 0u;
  }
  if (gtid == 0) ctl->cnt[0] = 1ull;
  if (!grid_barrier(ctl, p.timeout_ns, -1)) return;

  const long long nq = p.vec ? p.nnz >> 2 : 0; /* whole quads of pairs (16-byte aligned) */
  const int4 *I4 = reinterpret_cast<const int4 *>(p.I);
  const int4 *J4 = reinterpret_cast<const int4 *>(p.J);
  bool ovf = false;
  int d = 0;
  for (;; ++d) {
    const unsigned long long qn = __ldcg(&ctl->cnt[d % 3]);
    if (qn == 0) break;
    if (d >= p.max_levels) {
      if (gtid == 0) ctl->unfinished = 1;
      break;
    }
    if (gtid == 0) ctl->cnt[(d + 2) % 3] = 0ull;
    const unsigned *cur = p.fb[d % 3];
    unsigned *nxt = p.fb[(d + 1) % 3];
    unsigned *clr = p.fb[(d + 2) % 3];
    for (unsigned long long i = gtid; i < nwords; i += nthreads) clr[i] = 0u;
    unsigned taken = 0;
    for (long long q = (long long)gtid; q < nq; q += (long long)nthreads) {
      const int4 a = __ldcs(I4 + q);
      const int4 b = __ldcs(J4 + q);
      cooc_pair(p, d, a.x, b.x, cur, nxt, taken, ovf);
      cooc_pair(p, d, a.y, b.y, cur, nxt, taken, ovf);
      cooc_pair(p, d, a.z, b.z, cur, nxt, taken, ovf);
      cooc_pair(p, d, a.w, b.w, cur, nxt, taken, ovf);
    }
    for (long long k = 4 * nq + (long long)gtid; k < p.nnz; k += (long long)nthreads)
      cooc_pair(p, d, __ldg(p.I + k), __ldg(p.J + k), cur, nxt, taken, ovf);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) taken += __shfl_xor_sync(FULL, taken, o);
    if ((threadIdx.x & 31) == 0 && taken) atomicAdd(&ctl->cnt[(d + 1) % 3], (unsigned long long)taken);
    if (!grid_barrier(ctl, p.timeout_ns, d)) return;
  }
  if (__any_sync(FULL, ovf) && (threadIdx.x & 31) == 0) atomicOr(&ctl->sigma_overflow, 1);
  if (gtid == 0) ctl->levels = d;
}

/* bit 0 of *flag: some index outside [0, n) */
__global__ void cooc_check_kernel(const int *I, const int *J, long long nnz, int n, int *flag) {
  bool bad = false;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    const int a = __ldg(I + k), b = __ldg(J + k);
    bad |= a < 0 || a >= n || b < 0 || b >= n;
  }
  if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

}  // namespace

cudaError_t cooc_geometry(int device, LaunchGeom *out) {
  int sms = 0, coop = 0, per = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (e != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, cooc_bfs_kernel, kBlock, 0);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  if (per > 4) per = 4; /* a streaming pass: 32 warps per SM keep it in flight */
  out->block = kBlock;
  out->grid = sms * per;
  out->sms = sms;
  out->per_sm = per;
  return cudaSuccess;
}

cudaError_t cooc_launch(const CoocParams &p, const LaunchGeom &g, cudaStream_t s) {
  void *args[] = {const_cast<CoocParams *>(&p)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(cooc_bfs_kernel), dim3(g.grid),
                                     dim3(g.block), args, 0, s);
}

cudaError_t cooc_check(const int *I, const int *J, long long nnz, int n, int *d_flag,
                       cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_flag, 0, sizeof(int), s);
  if (e != cudaSuccess || nnz == 0) return e;
  const long long b = (nnz + 255) / 256;
  cooc_check_kernel<<<(unsigned)(b < 4096 ? b : 4096), 256, 0, s>>>(I, J, nnz, n, d_flag);
  return cudaGetLastError();
}

}  // namespace tbfs
