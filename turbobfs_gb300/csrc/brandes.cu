/*
 * brandes.cu -- betweenness centrality: the forward traversal of the engine
 * (depths S and path counts sigma, exactly what the reference computes) plus
 * Brandes' dependency sweep (U. Brandes, "A faster algorithm for betweenness
 * centrality", J. Math. Sociology 25(2), 2001):
 *
 *   delta[v] = sum over out-list entries v -> w with S[w] = S[v] + 1 of
 *              sigma[v] / sigma[w] * (1 + delta[w]),
 *   bc[v]   += delta[v] for every root s != v,
 * computed in the factored form delta[v] = sigma[v] * sum q[w] with
 * q[w] = (1 + delta[w]) / sigma[w], stored once w is final: one division
 * per vertex instead of one per entry, and one gather per entry.
 *
 * The sweep runs level by level from the deepest level up, as one
 * persistent cooperative launch per root with a grid barrier between levels.
 * Vertices are grouped by depth with a block-aggregated counting sort.
 * Every delta is a pull over the vertex's own out-list in a fixed order, so
 * the result does not depend on scheduling:
 *   out-degree < 32: one lane sums the terms in list order;
 *   otherwise the list is cut into segments of kSeg entries (one segment up
 *   to kSeg); in a segment, lane l sums the entries l, l+32, l+64, ... in
 *   order and the 32 partial sums meet in a butterfly (xor 16, 8, 4, 2, 1);
 *   the segments' sums are added in segment order.
 * A hub's segments are separate work items of the level, so a list of 10^5
 * entries is summed by tens of warps at once; its segment sums are combined
 * after a grid barrier.
 * All operations are correctly rounded IEEE double with no contraction into
 * fused multiply-adds, so a CPU restatement of the same order reproduces
 * every bit.  bc accumulates the roots in the order given.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "device_common.cuh"
#include "tbfs.h"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

using dev::FULL;
using dev::grid_barrier;

constexpr int kBlock = 256;
constexpr int kSmemLevels = 8192; /* levels counted in shared memory per block */
constexpr int kTile = 4096;       /* vertices per block of the counting sort   */
constexpr int kWarpDegree = 32;   /* out-degree from which a warp sums a vertex */
constexpr int kSeg = 2048;        /* entries per segment of a hub's list        */

struct __align__(128) SweepCtl {
  int status, timeout_level;
  unsigned work[4]; /* dynamic work counter of level d in work[d % 4] */
  int pad0[26];
  GridBarrier bar;
};

struct SweepParams {
  const int *rp, *jr;                /* out-lists (internal numbering)       */
  const int *S;                      /* depths of the forward traversal      */
  const unsigned long long *sig;     /* path counts                          */
  const int *list;                   /* vertices grouped by depth ...        */
  const int *off;                    /* ... level d at list[off[d], off[d+1]) */
  int levels;
  int root;                          /* caller numbering ...                 */
  const int *inv;                    /* ... mapped by inv (or null)          */
  double *q;                         /* n: (1 + delta[v]) / sigma[v], zero on entry */
  double *bc;                        /* n, accumulated                       */
  /* hubs (out-degree > kSeg) by list position i: segoff[i] (exclusive prefix
   * of their segment counts over positions), hoff[i] (of the hub flags);
   * hubpos[h] = position of hub h, seg_hub[s] = hub of segment s,
   * part[s] = sum of segment s */
  const int *segoff, *hoff, *hubpos, *seg_hub;
  double *part;
  /* vertices with 32 <= out-degree <= kSeg (a warp each): moff[i] exclusive
   * prefix of their flags over positions, medpos[m] = position of the m-th */
  const int *moff, *medpos;
  SweepCtl *ctl;
  long long timeout_ns;
};

/* v is final with the sum acc of its children's q: delta[v] to bc, q[v] */
__device__ __forceinline__ void finish(const SweepParams &p, int v, int root, double acc) {
  const double sv = (double)__ldg(p.sig + v);
  const double dv = __dmul_rn(sv, acc);
  p.q[v] = __ddiv_rn(__dadd_rn(1.0, dv), sv);
  if (v != root) p.bc[v] = __dadd_rn(p.bc[v], dv);
}

/* acc += q[w] of the entries k0, k0 + step, ... < e with S[w] = d + 1, in
 * that order; four entries' loads are issued before they are added */
__device__ __forceinline__ double sum_entries(const SweepParams &p, int d, int k0, int e,
                                              int step) {
  double acc = 0.0;
  int k = k0;
  for (; k + 3 * step < e; k += 4 * step) {
    int w[4];
    bool c[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = __ldg(p.jr + k + j * step);
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j] = __ldg(p.S + w[j]) == d + 1;
    double t[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) t[j] = c[j] ? __ldcg(p.q + w[j]) : 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (c[j]) acc = __dadd_rn(acc, t[j]);
  }
  for (; k < e; k += step) {
    const int w = __ldg(p.jr + k);
    if (__ldg(p.S + w) == d + 1) acc = __dadd_rn(acc, __ldcg(p.q + w));
  }
  return acc;
}

/* the terms of [b, e) summed lane-strided over the warp, then the butterfly;
 * every lane returns the same value (lane 0's order) */
__device__ __forceinline__ double warp_sum(const SweepParams &p, int d, int b, int e) {
  const int lane = threadIdx.x & 31;
  double acc = sum_entries(p, d, b + lane, e, 32);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(FULL, acc, o));
  return __shfl_sync(FULL, acc, 0);
}

__global__ void __launch_bounds__(kBlock) sweep_kernel(const SweepParams p) {
  const int lane = threadIdx.x & 31;
  const int root = p.inv ? __ldg(p.inv + p.root) : p.root;
  const unsigned gwarp = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * kBlock) >> 5;
  const unsigned gthread = blockIdx.x * kBlock + threadIdx.x;
  { /* the deepest level has no children: delta = 0, q = 1 / sigma */
    const int lo = __ldg(p.off + p.levels - 1), hi = __ldg(p.off + p.levels);
    for (int i = lo + (int)gthread; i < hi; i += (int)(gridDim.x * kBlock)) {
      const int v = __ldg(p.list + i);
      p.q[v] = __ddiv_rn(1.0, (double)__ldg(p.sig + v));
    }
    if (!grid_barrier(p.ctl, p.timeout_ns, p.levels - 1)) return;
  }
  for (int d = p.levels - 2; d >= 0; --d) {
    const int lo = __ldg(p.off + d), hi = __ldg(p.off + d + 1);
    const int s_lo = __ldg(p.segoff + lo), s_hi = __ldg(p.segoff + hi);
    const int h_lo = __ldg(p.hoff + lo), h_hi = __ldg(p.hoff + hi);
    const int m_lo = __ldg(p.moff + lo), m_hi = __ldg(p.moff + hi);
    const unsigned ns = (unsigned)(s_hi - s_lo), nm = (unsigned)(m_hi - m_lo);
    const unsigned nch = (unsigned)(hi - lo + 31) / 32u;
    const unsigned items = ns + nm + nch;
    /* work counter of level d-2 (last used at level d+2) */
    if (gthread == 0) p.ctl->work[(d + 2) & 3] = 0u;
    /* items, the long ones first: the hubs' segments, then the vertices a
     * warp sums, then chunks of 32 positions whose short lists one lane
     * each sums.  The first item of a warp is static, the rest claimed. */
    unsigned it = gwarp;
    while (it < items) {
      if (it < ns) { /* segment sg of a hub */
        const int sg = s_lo + (int)it;
        const int i = __ldg(p.hubpos + __ldg(p.seg_hub + sg));
        const int v = __ldg(p.list + i);
        const int b = __ldg(p.rp + v) + (sg - __ldg(p.segoff + i)) * kSeg;
        const int e = min(b + kSeg, __ldg(p.rp + v + 1));
        const double acc = warp_sum(p, d, b, e);
        if (lane == 0) p.part[sg] = acc;
      } else if (it < ns + nm) { /* a one-segment list, the whole warp */
        const int v = __ldg(p.list + __ldg(p.medpos + m_lo + (int)(it - ns)));
        const double acc = warp_sum(p, d, __ldg(p.rp + v), __ldg(p.rp + v + 1));
        if (lane == 0) finish(p, v, root, acc);
      } else { /* short lists, one lane each */
        const int i = lo + (int)(it - ns - nm) * 32 + lane;
        if (i < hi) {
          const int v = __ldg(p.list + i);
          const int b = __ldg(p.rp + v), e = __ldg(p.rp + v + 1);
          if (e - b < kWarpDegree) finish(p, v, root, sum_entries(p, d, b, e, 1));
        }
      }
      if (items <= nwarps) break;
      unsigned nxt = 0;
      if (lane == 0) nxt = nwarps + atomicAdd(&p.ctl->work[d & 3], 1u);
      it = __shfl_sync(FULL, nxt, 0);
    }
    if (h_hi > h_lo) { /* the hubs of level d: their segments in order */
      if (!grid_barrier(p.ctl, p.timeout_ns, d)) return;
      for (unsigned t = gthread; t < (unsigned)(h_hi - h_lo); t += gridDim.x * kBlock) {
        const int i = __ldg(p.hubpos + h_lo + (int)t);
        const int v = __ldg(p.list + i);
        const int s0 = __ldg(p.segoff + i), s1 = __ldg(p.segoff + i + 1);
        double acc = __ldcg(p.part + s0);
        for (int sg = s0 + 1; sg < s1; ++sg) acc = __dadd_rn(acc, __ldcg(p.part + sg));
        finish(p, v, root, acc);
      }
    }
    if (!grid_barrier(p.ctl, p.timeout_ns, d)) return;
  }
}

/* segs[i] = segments of the vertex at list position i (0 unless a hub),
 * flag[i] = it is a hub, mflag[i] = a warp sums its list; for i < *cnt (the
 * reached vertices), 0 up to len */
__global__ void hub_count_kernel(const int *list, const int *rp, const int *cnt, int len,
                                 int *segs, int *flag, int *mflag) {
  const int c = *cnt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
    int h = 0, sg = 0, m = 0;
    if (i < c) {
      const int v = list[i];
      const int deg = rp[v + 1] - rp[v];
      h = deg > kSeg ? 1 : 0;
      sg = h ? (deg + kSeg - 1) / kSeg : 0;
      m = deg >= kWarpDegree && deg <= kSeg ? 1 : 0;
    }
    segs[i] = sg;
    flag[i] = h;
    mflag[i] = m;
  }
}

/* medpos[moff[i]] = i for the positions a warp sums */
__global__ void med_fill_kernel(const int *moff, const int *cnt, int *medpos) {
  const int c = *cnt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c; i += gridDim.x * blockDim.x)
    if (moff[i + 1] != moff[i]) medpos[moff[i]] = i;
}

/* hubpos[hoff[i]] = i and seg_hub[s] = hoff[i] for the hubs' segments */
__global__ void hub_fill_kernel(const int *segoff, const int *hoff, const int *cnt,
                                int *hubpos, int *seg_hub) {
  const int c = *cnt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c; i += gridDim.x * blockDim.x) {
    const int h = hoff[i];
    if (hoff[i + 1] == h) continue;
    hubpos[h] = i;
    for (int sg = segoff[i]; sg < segoff[i + 1]; ++sg) seg_hub[sg] = h;
  }
}

/* ---- vertices grouped by depth (counting sort, block-aggregated) ---- */

/* counts[d] = vertices at depth d */
__global__ void level_count_kernel(const int *S, int n, int levels, int *counts) {
  __shared__ int h[kSmemLevels];
  const bool local = levels <= kSmemLevels;
  if (local)
    for (int d = threadIdx.x; d < levels; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kTile;
  for (int j = threadIdx.x; j < kTile; j += blockDim.x) {
    const long long v = base + j;
    if (v >= n) break;
    const int d = S[v];
    if (d < 0) continue;
    if (local)
      atomicAdd(&h[d], 1);
    else
      atomicAdd(&counts[d], 1);
  }
  __syncthreads();
  if (local)
    for (int d = threadIdx.x; d < levels; d += blockDim.x)
      if (h[d]) atomicAdd(&counts[d], h[d]);
}

/* list[...] = vertices by depth; fill[d] starts at the exclusive prefix */
__global__ void level_fill_kernel(const int *S, int n, int levels, int *fill, int *list) {
  __shared__ int h[kSmemLevels];
  const bool local = levels <= kSmemLevels;
  if (local)
    for (int d = threadIdx.x; d < levels; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kTile;
  if (local) {
    for (int j = threadIdx.x; j < kTile; j += blockDim.x) {
      const long long v = base + j;
      if (v >= n) break;
      const int d = S[v];
      if (d >= 0) atomicAdd(&h[d], 1);
    }
    __syncthreads();
    /* reserve this block's range of every level, then hand out positions */
    for (int d = threadIdx.x; d < levels; d += blockDim.x)
      if (h[d]) h[d] = atomicAdd(&fill[d], h[d]);
    __syncthreads();
    for (int j = threadIdx.x; j < kTile; j += blockDim.x) {
      const long long v = base + j;
      if (v >= n) break;
      const int d = S[v];
      if (d >= 0) list[atomicAdd(&h[d], 1)] = (int)v;
    }
  } else {
    for (int j = threadIdx.x; j < kTile; j += blockDim.x) {
      const long long v = base + j;
      if (v >= n) break;
      const int d = S[v];
      if (d >= 0) list[atomicAdd(&fill[d], 1)] = (int)v;
    }
  }
}

/* out[j] = in[inv[j]] (or in[j]) */
__global__ void gather_double_kernel(const double *in, const int *inv, int n, double *out) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) out[j] = in[inv ? inv[j] : j];
}

}  // namespace
}  // namespace tbfs

using tbfs::SweepCtl;
using tbfs::SweepParams;

namespace {

tbfs_status bfail(cudaError_t e, const char *what) {
  tbfs_set_error("tbfs_brandes: %s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
}

#define BTRY(call, what)                            \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return bfail(e_, what);  \
  } while (0)

struct Scratch {
  int *S = nullptr, *list = nullptr, *off = nullptr, *fill = nullptr;
  int *segoff = nullptr, *hoff = nullptr, *hubpos = nullptr, *seg_hub = nullptr;
  int *moff = nullptr, *medpos = nullptr;
  int *partial = nullptr; /* scan scratch */
  double *part = nullptr;
  unsigned long long *sig = nullptr;
  double *delta = nullptr, *bc = nullptr, *out = nullptr;
  SweepCtl *ctl = nullptr;
  tbfs::BfsCtl *fctl_host = nullptr;
  SweepCtl *ctl_host = nullptr;
  ~Scratch() {
    cudaFree(S);
    cudaFree(list);
    cudaFree(off);
    cudaFree(fill);
    cudaFree(segoff);
    cudaFree(hoff);
    cudaFree(hubpos);
    cudaFree(seg_hub);
    cudaFree(moff);
    cudaFree(medpos);
    cudaFree(part);
    cudaFree(partial);
    cudaFree(sig);
    cudaFree(delta);
    cudaFree(bc);
    cudaFree(out);
    cudaFree(ctl);
    if (fctl_host) cudaFreeHost(fctl_host);
    if (ctl_host) cudaFreeHost(ctl_host);
  }
};

}  // namespace

extern "C" tbfs_status tbfs_brandes(tbfs_graph *g, const int32_t *roots, int32_t k,
                                    const tbfs_options *opt, double *bc, int32_t *overflow) {
  tbfs_options o;
  tbfs_options_init(&o);
  if (opt) o = *opt;
  if (!g || k < 0 || (k > 0 && !roots) || !bc) {
    tbfs_set_error("tbfs_brandes: null graph, roots or bc, or k < 0");
    return TBFS_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) {
      tbfs_set_error("tbfs_brandes: root %d (index %d) outside [0, n)", roots[i], i);
      return TBFS_ERR_INVALID_ARG;
    }
  BTRY(cudaSetDevice(g->device), "cudaSetDevice");
  cudaStream_t s = (cudaStream_t)o.stream;
  const size_t n = (size_t)g->n;
  Scratch w;
  BTRY(cudaMalloc(&w.S, n * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.sig, n * sizeof(unsigned long long)), "alloc");
  BTRY(cudaMalloc(&w.list, n * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.off, (n + 2) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.fill, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.segoff, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.hoff, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.hubpos, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.moff, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.medpos, (n + 1) * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.partial, (size_t)tbfs::scan_partials((long long)n + 2) * sizeof(int)),
       "alloc");
  /* segments: each hub has deg > kSeg, so sum of ceil(deg / kSeg) < 2 nnz / kSeg + 1 */
  const size_t seg_cap = (size_t)(2 * g->nnz / tbfs::kSeg + 1);
  BTRY(cudaMalloc(&w.part, seg_cap * sizeof(double)), "alloc");
  BTRY(cudaMalloc(&w.seg_hub, seg_cap * sizeof(int)), "alloc");
  BTRY(cudaMalloc(&w.delta, n * sizeof(double)), "alloc");
  BTRY(cudaMalloc(&w.bc, n * sizeof(double)), "alloc");
  BTRY(cudaMalloc(&w.ctl, sizeof(SweepCtl)), "alloc");
  BTRY(cudaMallocHost(&w.fctl_host, sizeof(tbfs::BfsCtl)), "alloc");
  BTRY(cudaMemsetAsync(w.bc, 0, n * sizeof(double), s), "clear");
  /* grid of the sweep: all SMs, as occupancy allows (cooperative) */
  int sms = 0, per = 0;
  BTRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device), "attribute");
  BTRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tbfs::sweep_kernel, tbfs::kBlock, 0),
       "occupancy");
#ifndef TBFS_SWEEP_PER_SM
#define TBFS_SWEEP_PER_SM 4 /* 32 registers: 4 CTAs of 256 per SM measured 11 % faster than 2 */
#endif
  if (per > TBFS_SWEEP_PER_SM) per = TBFS_SWEEP_PER_SM;
  const unsigned grid = (unsigned)(sms * (per > 0 ? per : 1));
  const unsigned tiles = (unsigned)((n + tbfs::kTile - 1) / tbfs::kTile);
  const long long timeout = o.timeout_ns > 0 ? o.timeout_ns : 4000000000LL;
  int32_t ovf_roots = 0;
  tbfs_options fo = o;
  fo.want_sigma = 1;
  fo.outputs_on_device = 1;
  fo.level_trace = nullptr;
  fo.level_trace_cap = 0;
  for (int32_t r = 0; r < k; ++r) {
    tbfs_status st = tbfs::forward_internal(g, roots[r], fo, w.S, w.sig, s, w.fctl_host);
    if (st != TBFS_OK) return st;
    BTRY(cudaStreamSynchronize(s), "forward traversal");
    const tbfs::BfsCtl &fc = *w.fctl_host;
    if (fc.status != 0) {
      tbfs_set_error("tbfs_brandes: forward traversal: grid barrier wait exceeded its budget");
      return TBFS_ERR_TIMEOUT;
    }
    if (fc.sigma_overflow) ++ovf_roots;
    const int levels = fc.levels;
    if (levels < 2) continue; /* an isolated root: no dependencies */
    /* vertices by depth */
    BTRY(cudaMemsetAsync(w.off, 0, ((size_t)levels + 1) * sizeof(int), s), "clear");
    tbfs::level_count_kernel<<<tiles, tbfs::kBlock, 0, s>>>(w.S, g->n, levels, w.off);
    BTRY(cudaGetLastError(), "level count");
    BTRY(tbfs::exclusive_scan_ws(w.off, (long long)levels + 1, w.off, w.partial, s),
         "level prefix");
    BTRY(cudaMemcpyAsync(w.fill, w.off, (size_t)levels * sizeof(int), cudaMemcpyDeviceToDevice, s),
         "fill pointers");
    tbfs::level_fill_kernel<<<tiles, tbfs::kBlock, 0, s>>>(w.S, g->n, levels, w.fill, w.list);
    BTRY(cudaGetLastError(), "level fill");
    /* hubs: segment counts and flags by list position (positions < off[levels],
     * the reached vertices), their prefixes, the hub and segment maps */
    const unsigned cgrid = (unsigned)((n + 1 + 255) / 256);
    tbfs::hub_count_kernel<<<cgrid, 256, 0, s>>>(w.list, g->rp, w.off + levels, g->n + 1,
                                                 w.segoff, w.hoff, w.moff);
    BTRY(cudaGetLastError(), "hub count");
    BTRY(tbfs::exclusive_scan_ws(w.segoff, (long long)n + 1, w.segoff, w.partial, s),
         "segment prefix");
    BTRY(tbfs::exclusive_scan_ws(w.hoff, (long long)n + 1, w.hoff, w.partial, s), "hub prefix");
    BTRY(tbfs::exclusive_scan_ws(w.moff, (long long)n + 1, w.moff, w.partial, s), "warp prefix");
    tbfs::med_fill_kernel<<<cgrid, 256, 0, s>>>(w.moff, w.off + levels, w.medpos);
    BTRY(cudaGetLastError(), "warp positions");
    tbfs::hub_fill_kernel<<<cgrid, 256, 0, s>>>(w.segoff, w.hoff, w.off + levels, w.hubpos,
                                                w.seg_hub);
    BTRY(cudaGetLastError(), "hub fill");
    BTRY(cudaMemsetAsync(w.delta, 0, n * sizeof(double), s), "clear");
    BTRY(cudaMemsetAsync(w.ctl, 0, sizeof(SweepCtl), s), "clear");
    SweepParams p;
    p.rp = g->rp;
    p.jr = g->jr;
    p.S = w.S;
    p.sig = w.sig;
    p.list = w.list;
    p.off = w.off;
    p.levels = levels;
    p.root = roots[r];
    p.inv = g->inv;
    p.q = w.delta;
    p.bc = w.bc;
    p.segoff = w.segoff;
    p.hoff = w.hoff;
    p.hubpos = w.hubpos;
    p.seg_hub = w.seg_hub;
    p.moff = w.moff;
    p.medpos = w.medpos;
    p.part = w.part;
    p.ctl = w.ctl;
    p.timeout_ns = timeout;
    void *args[] = {&p};
    BTRY(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(tbfs::sweep_kernel), dim3(grid),
                                     dim3(tbfs::kBlock), args, 0, s),
         "dependency sweep");
    BTRY(cudaStreamSynchronize(s), "dependency sweep");
    SweepCtl sc;
    BTRY(cudaMemcpy(&sc, w.ctl, sizeof(sc), cudaMemcpyDeviceToHost), "read sweep status");
    if (sc.status != 0) {
      tbfs_set_error("tbfs_brandes: sweep: grid barrier wait exceeded its budget");
      return TBFS_ERR_TIMEOUT;
    }
  }
  /* results in the caller's numbering */
  double *dst = bc;
  if (!o.outputs_on_device) {
    BTRY(cudaMalloc(&w.out, n * sizeof(double)), "alloc");
    dst = w.out;
  }
  tbfs::gather_double_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w.bc, g->inv, g->n, dst);
  BTRY(cudaGetLastError(), "gather");
  if (!o.outputs_on_device)
    BTRY(cudaMemcpyAsync(bc, w.out, n * sizeof(double), cudaMemcpyDeviceToHost, s), "copy bc");
  BTRY(cudaStreamSynchronize(s), "results");
  if (overflow) *overflow = ovf_roots;
  return TBFS_OK;
}
