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
 * The sweep runs level by level from the deepest level up, in one persistent
 * cooperative launch for up to kMaxSweepRoots roots at once: step D works on
 * level D of every root whose traversal reached that deep, so the roots share
 * the grid barriers and fill the GPU where one root's level would not.
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
 * every bit.  Each root's delta is kept and bc adds them up after the sweep,
 * in the order of the roots given.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <vector>

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

constexpr int kMaxSweepRoots = 32; /* roots per sweep launch (one lane each in the plan) */

/* one root's arrays (internal numbering) */
struct RootSweep {
  const int *S;                      /* depths of the forward traversal      */
  const unsigned long long *sig;     /* path counts                          */
  const int *list;                   /* vertices grouped by depth ...        */
  const int *off;                    /* ... level d at list[off[d], off[d+1]) */
  int levels;
  int root;                          /* internal id of the root               */
  double *q;                         /* (1 + delta[v]) / sigma[v]             */
  double *dl;                        /* delta[v] (0 at the root), zero on entry */
  /* hubs (out-degree > kSeg) by list position i: segoff[i] (exclusive prefix
   * of their segment counts over positions), hoff[i] (of the hub flags);
   * hubpos[h] = position of hub h, seg_hub[s] = hub of segment s,
   * part[s] = sum of segment s */
  const int *segoff, *hoff, *hubpos, *seg_hub;
  double *part;
  /* vertices with 32 <= out-degree <= kSeg (a warp each): moff[i] exclusive
   * prefix of their flags over positions, medpos[m] = position of the m-th */
  const int *moff, *medpos;
};

struct SweepParams {
  const int *rp, *jr; /* out-lists (internal numbering) */
  const RootSweep *rs;
  int k;              /* roots of the launch            */
  int dmax;           /* largest number of levels       */
  SweepCtl *ctl;
  long long timeout_ns;
};

/* v is final with the sum acc of its children's q: its delta, q[v] */
__device__ __forceinline__ void finish(const RootSweep &R, int v, double acc) {
  const double sv = (double)__ldg(R.sig + v);
  const double dv = __dmul_rn(sv, acc);
  R.q[v] = __ddiv_rn(__dadd_rn(1.0, dv), sv);
  if (v != R.root) R.dl[v] = dv;
}

/* acc += q[w] of the entries k0, k0 + step, ... < e with S[w] = d + 1, in
 * that order; four entries' loads are issued before they are added */
__device__ __forceinline__ double sum_entries(const SweepParams &p, const RootSweep &R, int d,
                                              int k0, int e, int step) {
  double acc = 0.0;
  int k = k0;
  for (; k + 3 * step < e; k += 4 * step) {
    int w[4];
    bool c[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = __ldg(p.jr + k + j * step);
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j] = __ldg(R.S + w[j]) == d + 1;
    double t[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) t[j] = c[j] ? __ldcg(R.q + w[j]) : 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (c[j]) acc = __dadd_rn(acc, t[j]);
  }
  for (; k < e; k += step) {
    const int w = __ldg(p.jr + k);
    if (__ldg(R.S + w) == d + 1) acc = __dadd_rn(acc, __ldcg(R.q + w));
  }
  return acc;
}

/* the terms of [b, e) summed lane-strided over the warp, then the butterfly;
 * every lane returns the same value (lane 0's order) */
__device__ __forceinline__ double warp_sum(const SweepParams &p, const RootSweep &R, int d, int b,
                                           int e) {
  const int lane = threadIdx.x & 31;
  double acc = sum_entries(p, R, d, b + lane, e, 32);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(FULL, acc, o));
  return __shfl_sync(FULL, acc, 0);
}

/* Items of step D for root R: hub segments, lists a warp sums, chunks of 32
 * positions of short lists -- or, at the root's deepest level, chunks of 32
 * positions whose q = 1 / sigma (no children).  cnt[0..3]: segments, warp
 * lists, chunks, hubs to combine afterwards. */
__device__ __forceinline__ void step_counts(const RootSweep &R, int D, unsigned (&cnt)[4]) {
  cnt[0] = cnt[1] = cnt[2] = cnt[3] = 0u;
  if (D >= R.levels) return;
  const int lo = __ldg(R.off + D), hi = __ldg(R.off + D + 1);
  cnt[2] = (unsigned)(hi - lo + 31) / 32u;
  if (D == R.levels - 1) return;
  cnt[0] = (unsigned)(__ldg(R.segoff + hi) - __ldg(R.segoff + lo));
  cnt[1] = (unsigned)(__ldg(R.moff + hi) - __ldg(R.moff + lo));
  cnt[3] = (unsigned)(__ldg(R.hoff + hi) - __ldg(R.hoff + lo));
}

/* phase A item `it` (< ns + nm + nch) of root R at step D */
__device__ __forceinline__ void sweep_item(const SweepParams &p, const RootSweep &R, int D,
                                           unsigned it) {
  const int lane = threadIdx.x & 31;
  const int lo = __ldg(R.off + D), hi = __ldg(R.off + D + 1);
  if (D == R.levels - 1) { /* the root's deepest level: no children */
    const int i = lo + (int)it * 32 + lane;
    if (i < hi) {
      const int v = __ldg(R.list + i);
      R.q[v] = __ddiv_rn(1.0, (double)__ldg(R.sig + v));
    }
    return;
  }
  const int s_lo = __ldg(R.segoff + lo), m_lo = __ldg(R.moff + lo);
  const unsigned ns = (unsigned)(__ldg(R.segoff + hi) - s_lo);
  const unsigned nm = (unsigned)(__ldg(R.moff + hi) - m_lo);
  if (it < ns) { /* segment sg of a hub */
    const int sg = s_lo + (int)it;
    const int i = __ldg(R.hubpos + __ldg(R.seg_hub + sg));
    const int v = __ldg(R.list + i);
    const int b = __ldg(p.rp + v) + (sg - __ldg(R.segoff + i)) * kSeg;
    const int e = min(b + kSeg, __ldg(p.rp + v + 1));
    const double acc = warp_sum(p, R, D, b, e);
    if (lane == 0) R.part[sg] = acc;
  } else if (it < ns + nm) { /* a one-segment list, the whole warp */
    const int v = __ldg(R.list + __ldg(R.medpos + m_lo + (int)(it - ns)));
    const double acc = warp_sum(p, R, D, __ldg(p.rp + v), __ldg(p.rp + v + 1));
    if (lane == 0) finish(R, v, acc);
  } else { /* short lists, one lane each */
    const int i = lo + (int)(it - ns - nm) * 32 + lane;
    if (i < hi) {
      const int v = __ldg(R.list + i);
      const int b = __ldg(p.rp + v), e = __ldg(p.rp + v + 1);
      if (e - b < kWarpDegree) finish(R, v, sum_entries(p, R, D, b, e, 1));
    }
  }
}

/* smallest r with pre[r + 1] > x (pre[0] = 0, nondecreasing, k entries) */
__device__ __forceinline__ int root_of(const unsigned *pre, int k, unsigned x) {
  int lo = 0, hi = k - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pre[mid + 1] > x) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kBlock) sweep_kernel(const SweepParams p) {
  __shared__ unsigned s_pa[kMaxSweepRoots + 1], s_pb[kMaxSweepRoots + 1];
  __shared__ RootSweep s_rs[kMaxSweepRoots];
  const int lane = threadIdx.x & 31;
  const unsigned gwarp = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * kBlock) >> 5;
  const unsigned gthread = blockIdx.x * kBlock + threadIdx.x;
  const unsigned nthreads = gridDim.x * kBlock;
  for (int r = threadIdx.x; r < p.k; r += kBlock) s_rs[r] = p.rs[r];
  __syncthreads();
  for (int D = p.dmax - 1; D >= 0; --D) {
    /* the step's plan, identical in every CTA: per root, its phase-A items
     * and hubs to combine, as prefixes over the roots */
    if (threadIdx.x < 32) { /* lane r: root r's counts, then prefixes over the lanes */
      unsigned c[4] = {0u, 0u, 0u, 0u};
      if (lane < p.k) step_counts(s_rs[lane], D, c);
      const unsigned a = c[0] + c[1] + c[2], b = c[3];
      unsigned ia = a, ib = b;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned ta = __shfl_up_sync(FULL, ia, o), tb = __shfl_up_sync(FULL, ib, o);
        if (lane >= o) {
          ia += ta;
          ib += tb;
        }
      }
      if (lane < p.k) {
        s_pa[lane] = ia - a;
        s_pb[lane] = ib - b;
      }
      if (lane == p.k - 1) {
        s_pa[p.k] = ia;
        s_pb[p.k] = ib;
      }
    }
    /* work counter of step D-2 (last used at step D+2) */
    if (gthread == 0) p.ctl->work[(D + 2) & 3] = 0u;
    __syncthreads();
    const unsigned items = s_pa[p.k], hubs = s_pb[p.k];
    /* items: static first, then claimed; each root's long items come first */
    unsigned it = gwarp;
    while (it < items) {
      const int r = root_of(s_pa, p.k, it);
      sweep_item(p, s_rs[r], D, it - s_pa[r]);
      if (items <= nwarps) break;
      unsigned nxt = 0;
      if (lane == 0) nxt = nwarps + atomicAdd(&p.ctl->work[D & 3], 1u);
      it = __shfl_sync(FULL, nxt, 0);
    }
    if (hubs > 0) { /* the hubs of level D: their segment sums in order */
      if (!grid_barrier(p.ctl, p.timeout_ns, D)) return;
      for (unsigned t = gthread; t < hubs; t += nthreads) {
        const int r = root_of(s_pb, p.k, t);
        const RootSweep &R = s_rs[r];
        const int lo = __ldg(R.off + D);
        const int i = __ldg(R.hubpos + __ldg(R.hoff + lo) + (int)(t - s_pb[r]));
        const int v = __ldg(R.list + i);
        const int s0 = __ldg(R.segoff + i), s1 = __ldg(R.segoff + i + 1);
        double acc = __ldcg(R.part + s0);
        for (int sg = s0 + 1; sg < s1; ++sg) acc = __dadd_rn(acc, __ldcg(R.part + sg));
        finish(R, v, acc);
      }
    }
    if (!grid_barrier(p.ctl, p.timeout_ns, D)) return;
  }
}

/* bc[v] += dl_r[v] for the roots r of a launch, in order (dl is 0 where the
 * root did not reach v and at the root itself) */
__global__ void bc_add_kernel(double *bc, const double *dl, int k, int n) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    double x = bc[v];
    for (int r = 0; r < k; ++r) x = __dadd_rn(x, dl[(size_t)r * n + v]);
    bc[v] = x;
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

using tbfs::RootSweep;
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

/* the arrays of one root of a sweep launch (views into Scratch's pools) */
struct Slot {
  int *S = nullptr, *list = nullptr, *off = nullptr;
  int *segoff = nullptr, *hoff = nullptr, *hubpos = nullptr, *seg_hub = nullptr;
  int *moff = nullptr, *medpos = nullptr;
  unsigned long long *sig = nullptr;
  double *q = nullptr, *part = nullptr;
};

/* one allocation per kind of array for all slots: a call costs a dozen
 * cudaMalloc calls, not a dozen per root */
struct Scratch {
  std::vector<Slot> slots;
  int *ints = nullptr;                /* S, list, off, segoff, hoff, hubpos, moff, medpos, seg_hub */
  unsigned long long *sigs = nullptr;
  double *dbls = nullptr;             /* q, part */
  int *fill = nullptr, *partial = nullptr;
  double *dl = nullptr; /* K x n: each root's delta */
  double *bc = nullptr, *out = nullptr;
  RootSweep *rs = nullptr;
  SweepCtl *ctl = nullptr;
  tbfs::BfsCtl *fctl_host = nullptr;
  ~Scratch() {
    tbfs::dev_free(ints);
    tbfs::dev_free(sigs);
    tbfs::dev_free(dbls);
    tbfs::dev_free(fill);
    tbfs::dev_free(partial);
    tbfs::dev_free(dl);
    tbfs::dev_free(bc);
    tbfs::dev_free(out);
    tbfs::dev_free(rs);
    tbfs::dev_free(ctl);
    if (fctl_host) cudaFreeHost(fctl_host);
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
  /* roots per sweep launch: up to kMaxSweepRoots, fewer on large graphs
   * (each root holds about 60 n bytes while its launch runs) */
  int K = k < tbfs::kMaxSweepRoots ? (k > 0 ? k : 1) : tbfs::kMaxSweepRoots;
  while (K > 1 && (double)K * 64.0 * (double)n > 16e9) K /= 2;
  Scratch w;
  w.slots.resize((size_t)K);
  /* segments: each hub has deg > kSeg, so sum of ceil(deg / kSeg) < 2 nnz / kSeg + 1 */
  const size_t seg_cap = (size_t)(2 * g->nnz / tbfs::kSeg + 1);
  const size_t nI = n + 2; /* every int array of a slot: n + 2 entries */
  const size_t ints_per_slot = 8 * nI + seg_cap;
  const size_t dbls_per_slot = n + seg_cap;
  BTRY(tbfs::dev_alloc(&w.ints, (size_t)K * ints_per_slot * sizeof(int)), "alloc");
  BTRY(tbfs::dev_alloc(&w.sigs, (size_t)K * n * sizeof(unsigned long long)), "alloc");
  BTRY(tbfs::dev_alloc(&w.dbls, (size_t)K * dbls_per_slot * sizeof(double)), "alloc");
  for (int j = 0; j < K; ++j) {
    Slot &x = w.slots[(size_t)j];
    int *b = w.ints + (size_t)j * ints_per_slot;
    x.S = b;
    x.list = b + nI;
    x.off = b + 2 * nI;
    x.segoff = b + 3 * nI;
    x.hoff = b + 4 * nI;
    x.hubpos = b + 5 * nI;
    x.moff = b + 6 * nI;
    x.medpos = b + 7 * nI;
    x.seg_hub = b + 8 * nI;
    x.sig = w.sigs + (size_t)j * n;
    x.q = w.dbls + (size_t)j * dbls_per_slot;
    x.part = x.q + n;
  }
  BTRY(tbfs::dev_alloc(&w.fill, (n + 1) * sizeof(int)), "alloc");
  BTRY(tbfs::dev_alloc(&w.partial, (size_t)tbfs::scan_partials((long long)n + 2) * sizeof(int)),
       "alloc");
  BTRY(tbfs::dev_alloc(&w.dl, (size_t)K * n * sizeof(double)), "alloc");
  BTRY(tbfs::dev_alloc(&w.bc, n * sizeof(double)), "alloc");
  BTRY(tbfs::dev_alloc(&w.rs, (size_t)K * sizeof(RootSweep)), "alloc");
  BTRY(tbfs::dev_alloc(&w.ctl, sizeof(SweepCtl)), "alloc");
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
  const unsigned cgrid = (unsigned)((n + 1 + 255) / 256);
  const long long timeout = o.timeout_ns > 0 ? o.timeout_ns : 4000000000LL;
  int32_t ovf_roots = 0;
  tbfs_options fo = o;
  fo.want_sigma = 1;
  fo.outputs_on_device = 1;
  fo.level_trace = nullptr;
  fo.level_trace_cap = 0;
  std::vector<RootSweep> rs((size_t)K);
  for (int32_t r0 = 0; r0 < k; r0 += K) {
    const int kk = k - r0 < K ? k - r0 : K;
    int dmax = 0;
    BTRY(cudaMemsetAsync(w.dl, 0, (size_t)kk * n * sizeof(double), s), "clear");
    for (int j = 0; j < kk; ++j) {
      Slot &x = w.slots[(size_t)j];
      tbfs_status st = tbfs::forward_internal(g, roots[r0 + j], fo, x.S, x.sig, s, w.fctl_host);
      if (st != TBFS_OK) return st;
      BTRY(cudaStreamSynchronize(s), "forward traversal");
      const tbfs::BfsCtl &fc = *w.fctl_host;
      if (fc.status != 0) {
        tbfs_set_error("tbfs_brandes: forward traversal: grid barrier wait exceeded its budget");
        return TBFS_ERR_TIMEOUT;
      }
      if (fc.sigma_overflow) ++ovf_roots;
      const int levels = fc.levels;
      dmax = levels > dmax ? levels : dmax;
      /* vertices by depth */
      BTRY(cudaMemsetAsync(x.off, 0, ((size_t)levels + 1) * sizeof(int), s), "clear");
      tbfs::level_count_kernel<<<tiles, tbfs::kBlock, 0, s>>>(x.S, g->n, levels, x.off);
      BTRY(cudaGetLastError(), "level count");
      BTRY(tbfs::exclusive_scan_ws(x.off, (long long)levels + 1, x.off, w.partial, s),
           "level prefix");
      BTRY(cudaMemcpyAsync(w.fill, x.off, (size_t)levels * sizeof(int), cudaMemcpyDeviceToDevice,
                           s),
           "fill pointers");
      tbfs::level_fill_kernel<<<tiles, tbfs::kBlock, 0, s>>>(x.S, g->n, levels, w.fill, x.list);
      BTRY(cudaGetLastError(), "level fill");
      /* hubs and warp lists: flags by list position (positions < off[levels],
       * the reached vertices), their prefixes, the position maps */
      tbfs::hub_count_kernel<<<cgrid, 256, 0, s>>>(x.list, g->rp, x.off + levels, g->n + 1,
                                                   x.segoff, x.hoff, x.moff);
      BTRY(cudaGetLastError(), "hub count");
      BTRY(tbfs::exclusive_scan_ws(x.segoff, (long long)n + 1, x.segoff, w.partial, s),
           "segment prefix");
      BTRY(tbfs::exclusive_scan_ws(x.hoff, (long long)n + 1, x.hoff, w.partial, s), "hub prefix");
      BTRY(tbfs::exclusive_scan_ws(x.moff, (long long)n + 1, x.moff, w.partial, s),
           "warp prefix");
      tbfs::med_fill_kernel<<<cgrid, 256, 0, s>>>(x.moff, x.off + levels, x.medpos);
      BTRY(cudaGetLastError(), "warp positions");
      tbfs::hub_fill_kernel<<<cgrid, 256, 0, s>>>(x.segoff, x.hoff, x.off + levels, x.hubpos,
                                                  x.seg_hub);
      BTRY(cudaGetLastError(), "hub fill");
      RootSweep &R = rs[(size_t)j];
      R.S = x.S;
      R.sig = x.sig;
      R.list = x.list;
      R.off = x.off;
      R.levels = levels;
      R.root = g->inv ? -1 : roots[r0 + j]; /* internal id, filled below when renumbered */
      R.q = x.q;
      R.dl = w.dl + (size_t)j * n;
      R.segoff = x.segoff;
      R.hoff = x.hoff;
      R.hubpos = x.hubpos;
      R.seg_hub = x.seg_hub;
      R.part = x.part;
      R.moff = x.moff;
      R.medpos = x.medpos;
      if (g->inv)
        BTRY(cudaMemcpyAsync(&R.root, g->inv + roots[r0 + j], sizeof(int), cudaMemcpyDeviceToHost,
                             s),
             "root id");
    }
    BTRY(cudaStreamSynchronize(s), "sweep setup");
    BTRY(cudaMemcpyAsync(w.rs, rs.data(), (size_t)kk * sizeof(RootSweep), cudaMemcpyHostToDevice,
                         s),
         "sweep descriptors");
    BTRY(cudaMemsetAsync(w.ctl, 0, sizeof(SweepCtl), s), "clear");
    SweepParams p;
    p.rp = g->rp;
    p.jr = g->jr;
    p.rs = w.rs;
    p.k = kk;
    p.dmax = dmax;
    p.ctl = w.ctl;
    p.timeout_ns = timeout;
    void *args[] = {&p};
    BTRY(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(tbfs::sweep_kernel), dim3(grid),
                                     dim3(tbfs::kBlock), args, 0, s),
         "dependency sweep");
    tbfs::bc_add_kernel<<<cgrid, 256, 0, s>>>(w.bc, w.dl, kk, g->n);
    BTRY(cudaGetLastError(), "bc sums");
    SweepCtl sc;
    BTRY(cudaMemcpyAsync(&sc, w.ctl, sizeof(sc), cudaMemcpyDeviceToHost, s), "read sweep status");
    BTRY(cudaStreamSynchronize(s), "dependency sweep");
    if (sc.status != 0) {
      tbfs_set_error("tbfs_brandes: sweep: grid barrier wait exceeded its budget");
      return TBFS_ERR_TIMEOUT;
    }
  }
  /* results in the caller's numbering */
  double *dst = bc;
  if (!o.outputs_on_device) {
    BTRY(tbfs::dev_alloc(&w.out, n * sizeof(double)), "alloc");
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
