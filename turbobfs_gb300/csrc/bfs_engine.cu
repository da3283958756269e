/*
 * bfs_engine.cu -- one persistent, cooperatively launched kernel runs a whole
 * direction-optimizing BFS: every level is a phase separated by a
 * hand-written grid barrier, and the top-down / bottom-up decision is taken
 * on the device from counters the previous phase produced.  No host round
 * trip happens between levels.
 *
 * What it replaces in the reference: the per-level host loops of
 * TurboBFS_CSC_TD/bfsgputdcsc_sc.cu:95-119 (two launches and two event
 * syncs per level, host reads a managed flag), the bottom-up loop of
 * TurboBFS_CSC_BU/bfsgpubucsc_sc.cu:81-95, and the host-side switch of
 * TurboBFS_CSC_TDBU/bfsgputdbucsc_sc.cu:119-153 (managed float sizef).
 *
 * Level d (frontier F_d = vertices at depth d, held as a queue) does:
 *   top-down : edge-balanced push over the out-edges of F_d: an unvisited
 *              target is claimed with atomicCAS(S, -1, d+1) and appended to
 *              the next queue.
 *   bottom-up: every unvisited vertex scans its in-list and stops at the
 *              first in-neighbour with S == d (early exit).
 *   sigma    : sigma[v] for v in F_d is pulled once, in this same phase, as
 *              the sum of sigma[u] over in-list entries u with S[u] == d-1.
 *              These parents were finished one barrier earlier, so the pull
 *              never races with discovery, and bottom-up may stop early even
 *              when path counts are wanted.  For symmetric graphs the pull
 *              is fused into the top-down push (one read of each list).
 * sigma is exact in uint64 arithmetic; any sum that reaches 2^63 sets
 * ctl->sigma_overflow (overflow is reported, never rounded).
 *
 * Direction rule (device side; Beamer, Asanovic, Patterson, "Direction-
 * optimizing breadth-first search", SC 2012): leave top-down when the
 * frontier's out-edges exceed (unexplored edges)/alpha; return to top-down
 * when the frontier shrinks below n/beta.
 *
 * Memory model: S, sigma, the queues and the counters are written during
 * the kernel by other SMs, so they are read with ld.global.cg (L2) and never
 * through the non-coherent L1; read-only graph arrays use the L1 path.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "tbfs_internal.h"

namespace tbfs {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kBlock = 512;
enum { DIR_TD = 0, DIR_BU = 1 };

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile(const int *p) {
  return *reinterpret_cast<const volatile int *>(p);
}

/* a + b in uint64; flags sums that reach 2^63 or wrap */
__device__ __forceinline__ unsigned long long add_chk(unsigned long long a,
                                                      unsigned long long b, bool &ovf) {
  const unsigned long long s = a + b;
  if (s < a || (s >> 63)) ovf = true;
  return s;
}

/* Grid-wide barrier.  Thread 0 of every CTA arrives on a counter; the last
 * one resets it and bumps the generation word.  Every wait is bounded by
 * timeout_ns of wall time (globaltimer): on expiry the CTA records
 * TBFS_ERR_TIMEOUT and returns false, and so does every CTA that sees the
 * error word set, so the kernel always terminates. */
__device__ bool grid_barrier(BfsCtl *ctl, long long timeout_ns, int level) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned gen = ld_acquire_u32(&ctl->bar_gen);
    __threadfence();
    const unsigned prev = atomicAdd(&ctl->bar_arrive, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(&ctl->bar_arrive, 0u);
      __threadfence();
      st_release_u32(&ctl->bar_gen, gen + 1);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned spins = 0;
      while (ld_acquire_u32(&ctl->bar_gen) == gen) {
        if ((++spins & 31u) == 0) {
          if (ld_volatile(&ctl->status) != 0) {
            ok = 0;
            break;
          }
          if ((long long)(global_ns() - t0) > timeout_ns) {
            atomicCAS(&ctl->status, 0, (int)TBFS_ERR_TIMEOUT);
            atomicCAS(&ctl->timeout_level, 0, level + 2);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    if (ld_volatile(&ctl->status) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* Append the lanes with take=true to queue (q, e) of the next level:
 * one 64-bit atomic per warp reserves (count << 32 | out-edge sum), so the
 * queue position and the edge offset come from the same reservation and
 * e[] stays the exclusive prefix of out-degrees in queue order.  Must be
 * called by all 32 lanes. */
__device__ __forceinline__ void warp_append(bool take, int v, int deg, int *q, int *e,
                                            unsigned long long *ctr) {
  const unsigned m = __ballot_sync(FULL, take);
  if (m == 0) return;
  const int lane = threadIdx.x & 31;
  const int dv = take ? deg : 0;
  int incl = dv;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader)
    base = atomicAdd(ctr, ((unsigned long long)__popc(m) << 32) | (unsigned)total);
  base = __shfl_sync(FULL, base, leader);
  if (take) {
    const unsigned pos = (unsigned)(base >> 32) + __popc(m & lanemask_lt());
    q[pos] = v;
    e[pos] = (int)((unsigned)base + (unsigned)(incl - dv));
  }
}

/* Largest i in [0, qn) with e[i] <= target (e nondecreasing, e[0] = 0).
 * 32-ary search: each step narrows the range 32x with one load per lane. */
__device__ __forceinline__ int warp_find_owner(const int *e, unsigned qn, unsigned target) {
  const int lane = threadIdx.x & 31;
  unsigned lo = 0, hi = qn;
  while (hi - lo > 32) {
    const unsigned step = (hi - lo + 31) / 32;
    const unsigned pidx = lo + lane * step;
    const bool pred = pidx < hi && (unsigned)__ldcg(e + pidx) <= target;
    const unsigned m = __ballot_sync(FULL, pred);
    const unsigned last = 31 - __clz(m);
    lo = lo + last * step;
    const unsigned nhi = lo + step;
    hi = nhi < hi ? nhi : hi;
  }
  const unsigned pidx = lo + lane;
  const bool pred = pidx < hi && (unsigned)__ldcg(e + pidx) <= target;
  const unsigned m = __ballot_sync(FULL, pred);
  return (int)(lo + (31 - __clz(m)));
}

/* One warp processes the flattened out-edge range [E0, E1) of the queue
 * (qc, ec): warp-level load-balanced search over windows of 32 queue
 * entries, one edge per lane per round, coalesced reads of the lists.
 * PUSH: claim unvisited targets.  SIGMA: pull sigma from depth-(d-1)
 * neighbours (valid only when in-lists == out-lists). */
template <bool PUSH, bool SIGMA>
__device__ __forceinline__ void lbs_chunk(const BfsParams &p, int d, const int *qc,
                                          const int *ec, unsigned qn, unsigned qe,
                                          unsigned E0, unsigned E1, int *qx, int *ex,
                                          unsigned long long *ctr_next, bool &ovf) {
  const int lane = threadIdx.x & 31;
  const int *__restrict__ adjp = p.rp;
  const int *__restrict__ adji = p.jr;
  unsigned i0 = (unsigned)warp_find_owner(ec, qn, E0);
  unsigned pos = E0;
  while (pos < E1 && i0 < qn) {
    const unsigned idx = i0 + lane;
    int v = 0, a = 0;
    unsigned len = 0;
    if (idx < qn) {
      v = __ldcg(qc + idx);
      const unsigned eb = (unsigned)__ldcg(ec + idx);
      const unsigned ee = (idx + 1 < qn) ? (unsigned)__ldcg(ec + idx + 1) : qe;
      const unsigned b = eb > pos ? eb : pos;
      const unsigned en = ee < E1 ? ee : E1;
      if (en > b) {
        len = en - b;
        a = __ldg(adjp + v) + (int)(b - eb);
      }
    }
    unsigned incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const unsigned excl = incl - len;
    const unsigned total = __shfl_sync(FULL, incl, 31);
    unsigned long long acc = 0;
    for (unsigned base = 0; base < total; base += 32) {
      const unsigned t = base + lane;
      int k = 0; /* window entry owning edge t: largest k with excl_k <= t */
#pragma unroll
      for (int s = 16; s >= 1; s >>= 1) {
        const unsigned xs = __shfl_sync(FULL, excl, k + s);
        if (xs <= t) k += s;
      }
      const int ak = __shfl_sync(FULL, a, k);
      const unsigned xk = __shfl_sync(FULL, excl, k);
      const bool active = t < total;
      bool won = false;
      int u = 0;
      unsigned long long c = 0;
      if (active) {
        u = __ldg(adji + ak + (int)(t - xk));
        const int su = __ldcg(p.S + u);
        if (PUSH && su == -1) won = atomicCAS(p.S + u, -1, d + 1) == -1;
        if (SIGMA && su == d - 1) c = __ldcg(p.sigma + u);
      }
      if (PUSH) {
        int dg = 0;
        if (won) dg = __ldg(p.rp + u + 1) - __ldg(p.rp + u);
        warp_append(won, u, dg, qx, ex, ctr_next);
      }
      if (SIGMA) {
        unsigned long long s = c; /* segmented inclusive scan keyed by k */
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned long long sv = __shfl_up_sync(FULL, s, o);
          const int kv = __shfl_up_sync(FULL, k, o);
          if (lane >= o && kv == k) s = add_chk(s, sv, ovf);
        }
        /* window entry `lane` collects the segment sum at its last lane */
        const unsigned lo = excl > base ? excl : base;
        const unsigned hi0 = excl + len;
        const unsigned hi = hi0 < base + 32u ? hi0 : base + 32u;
        const int tail = hi > lo ? (int)(hi - 1u - base) : 0;
        const unsigned long long got = __shfl_sync(FULL, s, tail);
        if (hi > lo) acc = add_chk(acc, got, ovf);
      }
    }
    if (SIGMA && acc != 0) {
      const unsigned long long old = atomicAdd(p.sigma + v, acc);
      add_chk(old, acc, ovf);
    }
    pos += total;
    i0 += 32;
  }
}

/* sigma for F_d over in-lists, one warp per frontier vertex (used when the
 * graph is not symmetric, so the push lists cannot serve the pull). */
__device__ void sigma_pull_vertexwise(const BfsParams &p, int d, const int *qc,
                                      unsigned qn, unsigned gwarp, unsigned nwarps,
                                      bool &ovf) {
  const int lane = threadIdx.x & 31;
  for (unsigned i = gwarp; i < qn; i += nwarps) {
    const int v = __ldcg(qc + i);
    const int kb = __ldg(p.cp + v), ke = __ldg(p.cp + v + 1);
    unsigned long long s = 0;
    for (int k = kb + lane; k < ke; k += 32) {
      const int u = __ldg(p.ic + k);
      if (__ldcg(p.S + u) == d - 1) s = add_chk(s, __ldcg(p.sigma + u), ovf);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = add_chk(s, __shfl_xor_sync(FULL, s, o), ovf);
    if (lane == 0) p.sigma[v] = s;
  }
}

/* Bottom-up discovery: lane i of a warp owns vertex 32w+i; an unvisited
 * vertex scans its in-list until the first neighbour at depth d. */
__device__ void bu_discover(const BfsParams &p, int d, int *qx, int *ex,
                            unsigned long long *ctr, unsigned gwarp, unsigned nwarps) {
  const int lane = threadIdx.x & 31;
  const unsigned nwords = ((unsigned)p.n + 31u) >> 5;
  for (unsigned w = gwarp; w < nwords; w += nwarps) {
    const int v = (int)(w * 32u + (unsigned)lane);
    bool found = false;
    if (v < p.n && __ldcg(p.S + v) == -1) {
      int k = __ldg(p.cp + v);
      const int ke = __ldg(p.cp + v + 1);
      for (; k + 4 <= ke && !found; k += 4) { /* 4 independent gathers in flight */
        const int u0 = __ldg(p.ic + k), u1 = __ldg(p.ic + k + 1);
        const int u2 = __ldg(p.ic + k + 2), u3 = __ldg(p.ic + k + 3);
        const int s0 = __ldcg(p.S + u0), s1 = __ldcg(p.S + u1);
        const int s2 = __ldcg(p.S + u2), s3 = __ldcg(p.S + u3);
        found = (s0 == d) | (s1 == d) | (s2 == d) | (s3 == d);
      }
      for (; k < ke && !found; ++k) found = __ldcg(p.S + __ldg(p.ic + k)) == d;
      if (found) p.S[v] = d + 1;
    }
    const int dg = found ? (__ldg(p.rp + v + 1) - __ldg(p.rp + v)) : 0;
    warp_append(found, v, dg, qx, ex, ctr);
  }
}

__device__ __forceinline__ unsigned chunk_edges(unsigned qe, unsigned nwarps) {
  unsigned ch = (qe + nwarps - 1) / nwarps;
  ch = (ch + 31u) & ~31u;
  if (ch < 64u) ch = 64u;
  if (ch > 1024u) ch = 1024u;
  return ch;
}

__global__ void __launch_bounds__(kBlock) bfs_persistent_kernel(const BfsParams p) {
  const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned nthreads = gridDim.x * blockDim.x;
  const unsigned gwarp = gtid >> 5;
  const unsigned nwarps = nthreads >> 5;
  BfsCtl *ctl = p.ctl;
  const bool want_sigma = p.sigma != nullptr;

  /* init: S = -1, sigma = 0, root at depth 0 with one path */
  for (unsigned i = gtid; i < (unsigned)p.n; i += nthreads) {
    p.S[i] = (int)i == p.root ? 0 : -1;
    if (want_sigma) p.sigma[i] = (int)i == p.root ? 1ull : 0ull;
  }
  if (gtid == 0) {
    p.q0[0] = p.root;
    p.e0[0] = 0;
    const unsigned deg = (unsigned)(__ldg(p.rp + p.root + 1) - __ldg(p.rp + p.root));
    ctl->qctr[0] = (1ull << 32) | deg;
  }
  if (!grid_barrier(ctl, p.timeout_ns, -1)) return;

  int d = 0, dir = DIR_TD, td = 0, bu = 0;
  long long m_u = p.out_edges_total, visited = 0, edges = 0;
  unsigned prev_qn = 0;
  bool ovf = false;
  for (;;) {
    const unsigned long long cur = __ldcg(&ctl->qctr[d % 3]);
    const unsigned qn = (unsigned)(cur >> 32);
    const unsigned qe = (unsigned)cur;
    if (qn == 0) break;
    visited += qn;
    edges += qe;
    /* slot (d+2)%3 held F_{d-1}, read by every CTA before the last barrier;
     * clear it for F_{d+2}, which phase d+1 fills */
    if (gtid == 0) ctl->qctr[(d + 2) % 3] = 0ull;

    if (p.mode == TBFS_MODE_TOP_DOWN) {
      dir = DIR_TD;
    } else if (p.mode == TBFS_MODE_BOTTOM_UP) {
      dir = DIR_BU;
    } else if (dir == DIR_TD) {
      if ((double)qe > (double)m_u / (double)p.alpha) dir = DIR_BU;
      else m_u -= qe;
    } else if (qn < prev_qn && (double)qn <= (double)p.n / (double)p.beta) {
      dir = DIR_TD;
    }
    prev_qn = qn;

    const int *qc = (d & 1) ? p.q1 : p.q0;
    const int *ec = (d & 1) ? p.e1 : p.e0;
    int *qx = (d & 1) ? p.q0 : p.q1;
    int *ex = (d & 1) ? p.e0 : p.e1;
    unsigned long long *ctr_next = &ctl->qctr[(d + 1) % 3];
    const bool sig = want_sigma && d > 0;

    if (dir == DIR_TD) {
      ++td;
      const unsigned ch = chunk_edges(qe, nwarps);
      const unsigned nch = (qe + ch - 1) / ch;
      if (sig && p.symmetric) {
        for (unsigned c = gwarp; c < nch; c += nwarps) {
          const unsigned E0 = c * ch, E1 = E0 + ch < qe ? E0 + ch : qe;
          lbs_chunk<true, true>(p, d, qc, ec, qn, qe, E0, E1, qx, ex, ctr_next, ovf);
        }
      } else {
        for (unsigned c = gwarp; c < nch; c += nwarps) {
          const unsigned E0 = c * ch, E1 = E0 + ch < qe ? E0 + ch : qe;
          lbs_chunk<true, false>(p, d, qc, ec, qn, qe, E0, E1, qx, ex, ctr_next, ovf);
        }
        if (sig) sigma_pull_vertexwise(p, d, qc, qn, gwarp, nwarps, ovf);
      }
    } else {
      ++bu;
      if (sig) {
        if (p.symmetric) {
          const unsigned ch = chunk_edges(qe, nwarps);
          const unsigned nch = (qe + ch - 1) / ch;
          for (unsigned c = gwarp; c < nch; c += nwarps) {
            const unsigned E0 = c * ch, E1 = E0 + ch < qe ? E0 + ch : qe;
            lbs_chunk<false, true>(p, d, qc, ec, qn, qe, E0, E1, qx, ex, ctr_next, ovf);
          }
        } else {
          sigma_pull_vertexwise(p, d, qc, qn, gwarp, nwarps, ovf);
        }
      }
      bu_discover(p, d, qx, ex, ctr_next, gwarp, nwarps);
    }
    /* test hook: CTA 0 leaves without arriving; the others' waits expire */
    if (p.inject_barrier_skip > 0 && blockIdx.x == 0 && d == p.inject_barrier_skip - 1) return;
    if (!grid_barrier(ctl, p.timeout_ns, d)) break;
    ++d;
  }
  if (__any_sync(FULL, ovf) && (threadIdx.x & 31) == 0) atomicOr(&ctl->sigma_overflow, 1);
  if (gtid == 0) {
    ctl->levels = d;
    ctl->td_levels = td;
    ctl->bu_levels = bu;
    ctl->visited = visited;
    ctl->edges = edges;
  }
}

}  // namespace

cudaError_t bfs_geometry(int device, LaunchGeom *out) {
  int sms = 0, coop = 0, per = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (e != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bfs_persistent_kernel, kBlock, 0);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  out->block = kBlock;
  out->grid = sms * per;
  return cudaSuccess;
}

cudaError_t bfs_launch(const BfsParams &p, const LaunchGeom &g, cudaStream_t s) {
  void *args[] = {const_cast<BfsParams *>(&p)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(bfs_persistent_kernel),
                                     dim3(g.grid), dim3(g.block), args, 0, s);
}

}  // namespace tbfs
