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
 * Level d (frontier F_d = vertices at depth d, held as a queue) discovers
 * F_{d+1} either
 *   top-down : edge-balanced push over the out-edges of F_d; an unvisited
 *              target is claimed with atomicCAS(S, -1, d+1) and appended to
 *              the next queue, or
 *   bottom-up: every unvisited vertex scans its in-list and stops at the
 *              first in-neighbour with S == d (early exit).
 *
 * Path counts.  sigma[v] = sum of sigma[u] over the entries u->v with
 * S[u] = S[v]-1 (each such entry is a "parent edge").  The engine computes
 * sigma(F_{d+1}) wherever it is cheapest:
 *   - during a top-down discovery from F_d whose counts are final: every
 *     parent edge of F_{d+1} is examined by the push anyway, so each edge
 *     that lands on a vertex claimed at depth d+1 adds sigma[u] to it
 *     (no extra list reads);
 *   - otherwise (F_{d+1} was found bottom-up, which stops early) in the next
 *     phase, by either pulling over the lists of F_{d+1} or pushing from the
 *     lists of F_d -- whichever frontier has fewer edges.  The three most
 *     recent queues are kept, so F_d is still available then.
 * Counts are exact in uint64 arithmetic; any sum that reaches 2^63 sets
 * ctl->sigma_overflow (overflow is reported, never rounded).
 *
 * Edge-balanced expansion: each queue entry carries the vertex, the
 * exclusive prefix of out-degrees (its offset in the level's flattened edge
 * space) and the start of its list.  A warp takes a contiguous range of
 * flattened edges, stages 128 queue entries at a time in shared memory, and
 * every lane handles kEPT consecutive edges per round, so that many list
 * reads, then that many depth gathers, are in flight per lane.  On graphs
 * whose out-lists are all short (kShortList entries at most) the kernel
 * instance bfs_persistent_kernel<true> cuts small top-down levels into
 * items of kShortEntries whole queue entries instead, which need no owner
 * search (the chain of dependent L2 round trips is what a small level
 * costs); other graphs run the instance compiled without that path.
 *
 * Direction rule (device side; Beamer, Asanovic, Patterson, "Direction-
 * optimizing breadth-first search", SC 2012): leave top-down when the
 * frontier's out-edges exceed (unexplored edges)/alpha; return to top-down
 * when the frontier shrinks below n/beta.  The comparisons are in fp32:
 * every thread evaluates them at every level, and fp64 issues slowly on
 * this part (in fp64 they cost about 0.7 us per level).
 *
 * Memory model.  Queues and counters are read with ld.global.cg (L2).
 * Depth and path-count gathers use ordinary (L1-cacheable) loads: every
 * value a test acts on -- S == d-1, S == d, S == d+1 claimed earlier in this
 * phase only through an atomic's return value, sigma of a finished level --
 * was written before the last grid barrier, whose gpu-scope acquire makes it
 * visible to every later load of the CTA.  A plain load can return a stale
 * -1 for a vertex claimed during this phase; the engine then only attempts
 * an atomicCAS, whose return value is authoritative.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "tbfs_internal.h"

#ifndef TBFS_EPT
#define TBFS_EPT 6
#endif
#ifndef TBFS_BLOCK
#define TBFS_BLOCK 256
#endif
#ifndef TBFS_MIN_BLOCKS
#define TBFS_MIN_BLOCKS 4 /* 4 CTAs of 256 per SM: 64 registers (a small spill) */
#endif
#ifndef TBFS_SHORT_LEVELS
#define TBFS_SHORT_LEVELS 1 /* small top-down levels of short-list graphs: items of whole queue entries */
#endif
#ifndef TBFS_SHORT_CAS_FIRST
#define TBFS_SHORT_CAS_FIRST 1 /* aligned items claim with the CAS alone */
#endif
#ifndef TBFS_SPREAD_ITEMS
#define TBFS_SPREAD_ITEMS 1 /* static work items round-robin over the CTAs */
#endif
#ifndef TBFS_RED_PUSH
#define TBFS_RED_PUSH 1 /* pushes without the overflow check where a bound rules overflow out */
#endif

namespace tbfs {
namespace {

using dev::FULL;
using dev::add_chk;
using dev::smem_add_split;
using dev::global_ns;
using dev::grid_barrier;
using dev::warp_find_owner;
constexpr int kBlock = TBFS_BLOCK;
constexpr int kWarps = kBlock / 32;
constexpr int kWin = 128;          /* queue entries staged per warp window */
constexpr int kEPT = TBFS_EPT;     /* most consecutive edges per lane/round */
/* queue entries per item of a small level of a short-list graph: at most
 * 8 * kShortList = 128 edges, one round of at most 4 per lane */
constexpr unsigned kShortEntries = 8;
constexpr float kBuWordCost = 4.0f; /* a bitmap word of a bottom-up level, in list entries */
enum { DIR_TD = 0, DIR_BU = 1 };

/* what an expansion does with path counts */
enum SigMode {
  SIG_NONE = 0,     /* depths only                                          */
  SIG_PULL = 1,     /* entries gather sigma from neighbours at depth d-1    */
  SIG_PUSH_NEW = 2, /* entries add their sigma to targets claimed at d+1    */
  SIG_PUSH_AT = 3   /* entries add their sigma to targets at depth `tgt`    */
};

struct WarpWin {
  /* PULL: accumulator of the entry; PUSH: the entry's sigma -- as low and
   * high words in separate arrays, so that neighbouring entries fall in
   * different banks */
  unsigned lo[kWin], hi[kWin];
  int v[kWin];                  /* vertex of the entry                      */
  int a[kWin];                  /* list index of its first window edge      */
  unsigned s[kWin + 1];         /* window-relative start of its edges       */
};

/* Append, for every lane, the entries j < N with bit j of `take` set to the
 * next level's queue (q, e, a): one 64-bit atomic per warp reserves
 * (count << 32 | out-edge sum), so queue positions and edge offsets come from
 * the same reservation and e[] stays the exclusive prefix of out-degrees in
 * queue order.  Must be called by all 32 lanes. */
template <int N>
__device__ __forceinline__ void warp_append(unsigned take, const int (&vv)[N],
                                            const int (&dg)[N], const int (&ad)[N], int *q,
                                            int *e, int *a, unsigned long long *ctr) {
  const int lane = threadIdx.x & 31;
  const int cnt = __popc(take);
  int dsum = 0;
#pragma unroll
  for (int j = 0; j < N; ++j)
    if ((take >> j) & 1u) dsum += dg[j];
  int ic = cnt, id = dsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int tc = __shfl_up_sync(FULL, ic, o);
    const int td = __shfl_up_sync(FULL, id, o);
    if (lane >= o) {
      ic += tc;
      id += td;
    }
  }
  const int tot_c = __shfl_sync(FULL, ic, 31);
  if (tot_c == 0) return;
  const int tot_d = __shfl_sync(FULL, id, 31);
  unsigned long long base = 0;
  if (lane == 31)
    base = atomicAdd(ctr, ((unsigned long long)tot_c << 32) | (unsigned)tot_d);
  base = __shfl_sync(FULL, base, 31);
  unsigned pos = (unsigned)(base >> 32) + (unsigned)(ic - cnt);
  unsigned eo = (unsigned)base + (unsigned)(id - dsum);
#pragma unroll
  for (int j = 0; j < N; ++j) {
    if ((take >> j) & 1u) {
      q[pos] = vv[j];
      e[pos] = (int)eo;
      a[pos] = ad[j];
      ++pos;
      eo += (unsigned)dg[j];
    }
  }
}


/* A level's queue: entries i < qn with vertex q[i], edge offset e[i], list
 * start a[i]; qe is the total of its out-degrees. */
struct Queue {
  const int *q, *e, *a;
  unsigned qn, qe;
};

/* Output queue of the level being discovered. */
struct NextQueue {
  int *q, *e, *a;
  unsigned long long *ctr;
};

__device__ __forceinline__ bool bit_of(const unsigned *bm, int v) {
  return (bm[(unsigned)v >> 5] >> ((unsigned)v & 31u)) & 1u;
}

/* One warp expands the flattened out-edge range [E0, E1) of queue Q.
 * DISC: claim unvisited targets at depth d+1 into `nx` (and bitmap nb).
 * SIG: see SigMode (PULL is valid only when in-lists == out-lists; the push
 * modes walk the out-lists, which hold exactly the parent edges of their
 * targets).  Without DISC, membership of a neighbour in the level the mode
 * needs (d-1 for PULL, tgt for PUSH_AT) is read from bitmap tb, one bit per
 * vertex, instead of from S. */
template <bool DISC, int SIG, bool CHK = true, bool ALIGNED = false>
__device__ __forceinline__ void expand_chunk(const BfsParams &p, int d, int tgt, const Queue &Q,
                                             unsigned E0, unsigned E1, unsigned ept,
                                             const NextQueue &nx, const unsigned *tb,
                                             unsigned *nb, WarpWin &w, bool &ovf,
                                             unsigned first = 0, unsigned count = 0) {
  const int lane = threadIdx.x & 31;
  /* ALIGNED item: entries [first, first + count), all their edges, one
   * window; E0 = 0 and E1 = ~0u, so the window offsets below are the
   * entries' own edge offsets and no owner search is needed */
  constexpr bool aligned = ALIGNED;
  unsigned i0 = aligned ? first : warp_find_owner(Q.e, Q.qn, E0);
  unsigned pos = E0;
  while (pos < E1 && i0 < Q.qn) {
    unsigned nw = (Q.qn - i0) < (unsigned)kWin ? (Q.qn - i0) : (unsigned)kWin;
    if (aligned && count < nw) nw = count;
    for (unsigned k = lane; k < nw; k += 32) {
      const unsigned i = i0 + k;
      const unsigned eb = (unsigned)__ldcg(Q.e + i);
      const unsigned b = eb > pos ? eb : pos;
      const unsigned bc = b < E1 ? b : E1;
      const int v = __ldcg(Q.q + i);
      w.v[k] = v;
      w.a[k] = __ldcg(Q.a + i) + (int)(b - eb);
      w.s[k] = bc - pos;
      if (SIG == SIG_PULL) {
        w.lo[k] = 0u;
        w.hi[k] = 0u;
      }
      if ((SIG == SIG_PUSH_NEW || SIG == SIG_PUSH_AT) && !aligned) {
        const unsigned long long x = p.sigma[v];
        w.lo[k] = (unsigned)x;
        w.hi[k] = (unsigned)(x >> 32);
      }
    }
    if (lane == 0) {
      const unsigned ee = (i0 + nw < Q.qn) ? (unsigned)__ldcg(Q.e + i0 + nw) : Q.qe;
      w.s[nw] = (ee < E1 ? ee : E1) - pos;
    }
    __syncwarp();
    /* window edges t in [s[0], s[nw]): s[0] = 0 for an edge chunk, the
     * first entry's edge offset for an entry-aligned item */
    const unsigned t_beg = aligned ? w.s[0] : 0u, tot = w.s[nw];
    if (aligned) { /* one round when it fits: (edges + 31) / 32 per lane */
      const unsigned per = (tot - t_beg + 31u) / 32u;
      ept = per < 1u ? 1u : (per > ept ? ept : per);
    }
    const unsigned round = 32u * ept;
    for (unsigned base = t_beg; base < tot; base += round) {
      const unsigned t0 = base + (unsigned)lane * ept;
      const unsigned tend = t0 + ept < tot ? t0 + ept : tot;
      int u[kEPT], kk[kEPT];
      unsigned valid = 0;
#pragma unroll
      for (int j = 0; j < kEPT; ++j) {
        kk[j] = 0;
        u[j] = 0;
      }
      if (t0 < tot) {
        unsigned lo = 0, hi = nw - 1; /* largest k with s[k] <= t0 */
        while (lo < hi) {
          const unsigned mid = (lo + hi + 1) >> 1;
          if (w.s[mid] <= t0) lo = mid;
          else hi = mid - 1;
        }
        unsigned k = lo;
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          const unsigned t = t0 + j;
          if (t < tend) {
            while (w.s[k + 1] <= t) ++k;
            u[j] = w.a[k] + (int)(t - w.s[k]);
            kk[j] = (int)k;
            valid |= 1u << j;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kEPT; ++j) /* list reads, all in flight */
        if ((valid >> j) & 1u) u[j] = __ldg(p.jr + u[j]);
      /* an aligned item reads its entries' path counts with the list
       * entries instead of staging them first: one round trip fewer */
      unsigned long long xs[kEPT];
      if (aligned && SIG == SIG_PUSH_NEW) {
#pragma unroll
        for (int j = 0; j < kEPT; ++j) xs[j] = ((valid >> j) & 1u) ? p.sigma[w.v[kk[j]]] : 0ull;
      }
      int su[kEPT];   /* DISC: depth of the neighbour                        */
      unsigned in = 0; /* bit j: neighbour j is in the level the sigma mode needs */
      /* an aligned item may claim with the CAS alone: its return value is
       * the depth the plain read would have given */
      constexpr bool cas_first = aligned && TBFS_SHORT_CAS_FIRST;
      int ad[kEPT], dg[kEPT];
      if (DISC && cas_first) {
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          su[j] = -2;
          ad[j] = 0;
          dg[j] = 0;
          if ((valid >> j) & 1u) {
            su[j] = atomicCAS(p.S + u[j], -1, d + 1);
            ad[j] = __ldg(p.rp + u[j]);
            dg[j] = __ldg(p.rp + u[j] + 1) - ad[j];
          }
        }
      } else if (DISC) {
#pragma unroll
        for (int j = 0; j < kEPT; ++j) su[j] = ((valid >> j) & 1u) ? p.S[u[j]] : -2;
        if (SIG == SIG_PULL) {
#pragma unroll
          for (int j = 0; j < kEPT; ++j)
            if (su[j] == d - 1) in |= 1u << j;
        }
      } else {
        unsigned wd[kEPT];
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          su[j] = -2;
          wd[j] = ((valid >> j) & 1u) ? tb[(unsigned)u[j] >> 5] : 0u;
        }
#pragma unroll
        for (int j = 0; j < kEPT; ++j)
          if ((wd[j] >> ((unsigned)u[j] & 31u)) & 1u) in |= 1u << j;
      }
      unsigned hit = 0; /* PUSH_NEW: targets at depth d+1 after this edge */
      if (DISC) {
        unsigned take = 0;
        if (cas_first) {
#pragma unroll
          for (int j = 0; j < kEPT; ++j) {
            if (su[j] == -1) take |= 1u << j;
            else if (su[j] == d + 1) hit |= 1u << j;
          }
        } else {
#pragma unroll
          for (int j = 0; j < kEPT; ++j) {
            if (su[j] == -1) {
              const int old = atomicCAS(p.S + u[j], -1, d + 1);
              if (old == -1) take |= 1u << j;
              else if (old == d + 1) hit |= 1u << j;
            } else if (su[j] == d + 1) {
              hit |= 1u << j;
            }
          }
        }
        hit |= take;
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          if (!cas_first) {
            ad[j] = 0;
            dg[j] = 0;
          }
          if ((take >> j) & 1u) {
            if (!cas_first) {
              ad[j] = __ldg(p.rp + u[j]);
              dg[j] = __ldg(p.rp + u[j] + 1) - ad[j];
            }
            atomicOr(nb + ((unsigned)u[j] >> 5), 1u << ((unsigned)u[j] & 31u));
          }
        }
        warp_append<kEPT>(take, u, dg, ad, nx.q, nx.e, nx.a, nx.ctr);
      }
      if (SIG == SIG_PUSH_NEW || SIG == SIG_PUSH_AT) {
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          const bool add = SIG == SIG_PUSH_NEW ? ((hit >> j) & 1u) != 0 : ((in >> j) & 1u) != 0;
          if (add) {
            const unsigned long long x =
                aligned && SIG == SIG_PUSH_NEW
                    ? xs[j]
                    : ((unsigned long long)w.hi[kk[j]] << 32) | (unsigned long long)w.lo[kk[j]];
            if (CHK) add_chk(atomicAdd(p.sigma + u[j], x), x, ovf);
            else atomicAdd(p.sigma + u[j], x); /* result unused: a reduction, no round trip */
          }
        }
      }
      if (SIG == SIG_PULL) {
        unsigned long long c[kEPT]; /* path counts of the parents only */
#pragma unroll
        for (int j = 0; j < kEPT; ++j) c[j] = ((in >> j) & 1u) ? p.sigma[u[j]] : 0ull;
        unsigned long long run = 0;
        int rk = kk[0];
#pragma unroll
        for (int j = 0; j < kEPT; ++j) {
          if (kk[j] != rk) {
            if (run) smem_add_split(&w.lo[rk], &w.hi[rk], run, ovf);
            rk = kk[j];
            run = 0;
          }
          run = add_chk(run, c[j], ovf);
        }
        if (run) smem_add_split(&w.lo[rk], &w.hi[rk], run, ovf);
      }
    }
    __syncwarp();
    if (SIG == SIG_PULL) {
      for (unsigned k = lane; k < nw; k += 32) {
        const unsigned long long x = ((unsigned long long)w.hi[k] << 32) | (unsigned long long)w.lo[k];
        if (x) add_chk(atomicAdd(p.sigma + w.v[k], x), x, ovf);
      }
    }
    __syncwarp();
    if (aligned) break;
    pos += tot;
    i0 += nw;
  }
}

/* How one expansion of queue Q is cut into work items (edge chunks).
 * Small frontiers use fewer edges per lane (down to one), so their work is
 * spread over more warps and each lane's chain of dependent loads is short;
 * large frontiers use kEPT for memory-level parallelism.  About four chunks
 * per warp keep the dynamic scheduler balanced. */
struct ExpandPlan {
  unsigned ept, ch, nch;
};

__device__ __forceinline__ ExpandPlan plan_expand(unsigned qe, unsigned nwarps, unsigned max_ept) {
  ExpandPlan pl;
  const unsigned per_lane = (qe + 32u * nwarps - 1) / (32u * nwarps);
  pl.ept = per_lane < 1u ? 1u : (per_lane > max_ept ? max_ept : per_lane);
  const unsigned round = 32u * pl.ept;
  unsigned ch = (qe + 4u * nwarps - 1) / (4u * nwarps);
  ch = (ch + round - 1) / round * round;
  if (ch < round) ch = round;
  if (ch > 16u * round) ch = 16u * round;
  pl.ch = ch;
  pl.nch = (qe + ch - 1) / ch;
  return pl;
}

/* the expansions a phase can run (template instances of expand_chunk) */
enum ExpandKind {
  EX_NONE = 0,
  EX_DISC = 1,          /* discovery, depths only                 */
  EX_DISC_PUSH_NEW = 2, /* discovery + counts pushed to new targets */
  EX_DISC_PULL = 3,     /* discovery + counts of the entries pulled */
  EX_PUSH_AT = 4,       /* counts pushed to targets at depth tgt    */
  EX_PULL = 5           /* counts of the entries pulled             */
};

struct ExpandTask {
  int kind, tgt;
  Queue Q;
  const unsigned *tb;
  ExpandPlan pl;
  bool chk; /* pushes check every add for overflow */
};

__device__ __forceinline__ void run_expand_item(const BfsParams &p, int d, const ExpandTask &t,
                                                unsigned c, const NextQueue &nx, unsigned *nb,
                                                WarpWin &w, bool &ovf) {
  const unsigned E0 = c * t.pl.ch;
  const unsigned E1 = E0 + t.pl.ch < t.Q.qe ? E0 + t.pl.ch : t.Q.qe;
  switch (t.kind) {
    case EX_DISC:
      expand_chunk<true, SIG_NONE>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb, w, ovf);
      break;
    case EX_DISC_PUSH_NEW:
      if (t.chk)
        expand_chunk<true, SIG_PUSH_NEW>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb, w, ovf);
      else
        expand_chunk<true, SIG_PUSH_NEW, false>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb,
                                                w, ovf);
      break;
    case EX_DISC_PULL:
      expand_chunk<true, SIG_PULL>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb, w, ovf);
      break;
    case EX_PUSH_AT:
      if (t.chk)
        expand_chunk<false, SIG_PUSH_AT>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb, w, ovf);
      else
        expand_chunk<false, SIG_PUSH_AT, false>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb,
                                                w, ovf);
      break;
    case EX_PULL:
      expand_chunk<false, SIG_PULL>(p, d, t.tgt, t.Q, E0, E1, t.pl.ept, nx, t.tb, nb, w, ovf);
      break;
    default:
      break;
  }
}

/* One item of a small top-down level of a short-list graph: queue entries
 * [first, first + kShortEntries) with all their edges (ALIGNED expand_chunk:
 * no owner search). */
__device__ __forceinline__ void run_short_item(const BfsParams &p, int d, const ExpandTask &t, unsigned first,
                    unsigned max_ept, const NextQueue &nx, unsigned *nb, WarpWin &w, bool &ovf) {
  const unsigned ept = max_ept < 4u ? max_ept : 4u;
  if (t.kind == EX_DISC)
    expand_chunk<true, SIG_NONE, true, true>(p, d, 0, t.Q, 0u, ~0u, ept, nx, t.tb, nb, w, ovf,
                                             first, kShortEntries);
  else if (t.chk)
    expand_chunk<true, SIG_PUSH_NEW, true, true>(p, d, 0, t.Q, 0u, ~0u, ept, nx, t.tb, nb, w,
                                                 ovf, first, kShortEntries);
  else
    expand_chunk<true, SIG_PUSH_NEW, false, true>(p, d, 0, t.Q, 0u, ~0u, ept, nx, t.tb, nb, w,
                                                  ovf, first, kShortEntries);
}

/* Bottom-up discovery.  A warp takes kBuWords consecutive 32-vertex words
 * per iteration; lane i owns vertex 32*word+i of each, so the depth checks,
 * list bounds and the first gathers of all kBuWords vertices are in flight
 * together.  An unvisited vertex scans its in-list until the first
 * neighbour in F_d (bitmap cb); the scan advances every still-searching
 * vertex of the lane by one entry per step.  The warp owns its words of the
 * next level's bitmap nb and writes them whole. */
constexpr int kBuWords = 8;

__device__ void bu_tile(const BfsParams &p, int d, const NextQueue &nx, const unsigned *cb,
                        unsigned *nb, unsigned tile) {
  const int lane = threadIdx.x & 31;
  const unsigned nwords = ((unsigned)p.n + 31u) >> 5;
  {
    int v[kBuWords], k[kBuWords], ke[kBuWords];
    unsigned search = 0; /* bit j: vertex j unvisited and still searching */
#pragma unroll
    for (int j = 0; j < kBuWords; ++j) {
      v[j] = (int)((tile * kBuWords + j) * 32u + (unsigned)lane);
      k[j] = 0;
      ke[j] = 0;
      if (v[j] < p.n && p.S[v[j]] == -1) search |= 1u << j;
    }
#pragma unroll
    for (int j = 0; j < kBuWords; ++j)
      if ((search >> j) & 1u) {
        k[j] = __ldg(p.cp + v[j]);
        ke[j] = __ldg(p.cp + v[j] + 1);
      }
    unsigned found = 0;
    while (search) { /* two list entries per searching vertex per step */
      int u0[kBuWords], u1[kBuWords];
#pragma unroll
      for (int j = 0; j < kBuWords; ++j) {
        if (((search >> j) & 1u) && k[j] >= ke[j]) search &= ~(1u << j); /* list exhausted */
        const bool on = (search >> j) & 1u;
        u0[j] = on ? __ldg(p.ic + k[j]) : 0;
        u1[j] = (on && k[j] + 1 < ke[j]) ? __ldg(p.ic + k[j] + 1) : -1;
      }
#pragma unroll
      for (int j = 0; j < kBuWords; ++j) {
        if ((search >> j) & 1u) {
          if (bit_of(cb, u0[j]) || (u1[j] >= 0 && bit_of(cb, u1[j]))) {
            found |= 1u << j;
            search &= ~(1u << j);
          } else {
            k[j] += 2;
          }
        }
      }
    }
    int dg[kBuWords], ad[kBuWords];
#pragma unroll
    for (int j = 0; j < kBuWords; ++j) {
      dg[j] = 0;
      ad[j] = 0;
      if ((found >> j) & 1u) {
        p.S[v[j]] = d + 1;
        ad[j] = __ldg(p.rp + v[j]);
        dg[j] = __ldg(p.rp + v[j] + 1) - ad[j];
      }
    }
#pragma unroll
    for (int j = 0; j < kBuWords; ++j) {
      const unsigned word = __ballot_sync(FULL, (found >> j) & 1u);
      const unsigned wi = tile * kBuWords + j;
      if (lane == 0 && wi < nwords) nb[wi] = word;
    }
    warp_append<kBuWords>(found, v, dg, ad, nx.q, nx.e, nx.a, nx.ctr);
  }
}

template <bool SHORT>
__global__ void __launch_bounds__(kBlock, TBFS_MIN_BLOCKS) bfs_persistent_kernel(const BfsParams p) {
  __shared__ WarpWin s_win[kWarps];
  WarpWin &win = s_win[threadIdx.x >> 5];
  const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned nthreads = gridDim.x * blockDim.x;
  const unsigned nwarps = nthreads >> 5;
  BfsCtl *ctl = p.ctl;
  const bool want_sigma = p.sigma != nullptr;
  const int root = p.inv ? __ldg(p.inv + p.root) : p.root; /* internal numbering */

  /* init: S = -1, sigma = 0, root at depth 0 with one path; F_0 = {root} in
   * bitmap 0, the other bitmaps empty */
  for (unsigned i = gtid; i < (unsigned)p.n; i += nthreads) {
    p.S[i] = (int)i == root ? 0 : -1;
    if (want_sigma) p.sigma[i] = (int)i == root ? 1ull : 0ull;
  }
  const unsigned nwords = ((unsigned)p.n + 31u) >> 5;
  for (unsigned i = gtid; i < nwords; i += nthreads) {
    p.fb[0][i] = i == ((unsigned)root >> 5) ? 1u << ((unsigned)root & 31u) : 0u;
    p.fb[1][i] = 0u;
    p.fb[2][i] = 0u;
    p.fb[3][i] = 0u;
  }
  if (gtid == 0) {
    const int a = __ldg(p.rp + root);
    p.q[0][0] = root;
    p.e[0][0] = 0;
    p.a[0][0] = a;
    const unsigned deg = (unsigned)(__ldg(p.rp + root + 1) - a);
    ctl->qctr[0] = (1ull << 32) | deg;
  }
  if (!grid_barrier(ctl, p.timeout_ns, -1)) return;

  int d = 0, dir = DIR_TD, td = 0, bu = 0;
  long long m_u = p.out_edges_total, visited = 0, edges = 0;
  unsigned prev_qn = 0, prev_qe = 0;
  bool ovf = false, sig_ready = true; /* sigma(F_d) final at the start of phase d */
  bool done = false;
  /* Bound on the bits of the path counts of F_d: sigma(F_0) = 1, and a count
   * of F_{d+1} sums at most max-in-degree counts of F_d, so it has at most
   * deg_bits more bits.  Pushes into a level whose bound is at most 63 bits
   * cannot overflow and add without the check (a reduction whose result
   * is not waited for); so do pushes once an overflow has been recorded,
   * since the flag is per traversal. */
  int sig_bits = 1;
  for (;;) {
    const unsigned long long cur = __ldcg(&ctl->qctr[d % 3]);
    /* read with the counter, so that both loads are in flight together */
    const bool ovf_seen = TBFS_RED_PUSH && want_sigma && __ldcg(&ctl->sigma_overflow) != 0;
    const unsigned qn = (unsigned)(cur >> 32);
    const unsigned qe = (unsigned)cur;
    if (qn == 0) {
      done = true;
      break;
    }
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
      /* a bottom-up level also visits every vertex's bitmap word: without
       * that term, the tail of a deep graph (few unexplored edges left)
       * switched to bottom-up levels three times as costly as top-down ones */
      if ((float)qe * p.alpha > (float)m_u + kBuWordCost * (float)nwords) dir = DIR_BU;
      else m_u -= qe;
    } else if (qn < prev_qn && (float)qn * p.beta <= (float)p.n) {
      dir = DIR_TD;
    }
    if (gtid == 0 && p.trace && d < p.trace_cap - 1) {
      long long *rec = p.trace + 4 * (long long)d;
      rec[0] = (long long)global_ns();
      rec[1] = qn;
      rec[2] = qe;
      rec[3] = dir;
    }

    /* queues of levels d-1, d, d+1 rotate through three buffers */
    const int bc = d % 3, bn = (d + 1) % 3, bp = (d + 2) % 3;
    const Queue Qc = {p.q[bc], p.e[bc], p.a[bc], qn, qe};
    const Queue Qp = {p.q[bp], p.e[bp], p.a[bp], prev_qn, prev_qe};
    const NextQueue nx = {p.q[bn], p.e[bn], p.a[bn], &ctl->qctr[bn]};
    /* bitmaps: F_{d-1}, F_d read; F_{d+1} written; F_{d+2}'s cleared (its
     * previous contents, F_{d-2}, were last read in phase d-1) */
    const unsigned *bm_prev = p.fb[(d + 3) % 4];
    const unsigned *bm_cur = p.fb[d % 4];
    unsigned *bm_next = p.fb[(d + 1) % 4];
    unsigned *bm_clear = p.fb[(d + 2) % 4];
    for (unsigned i = gtid; i < nwords; i += nthreads) bm_clear[i] = 0u;
    /* work counter of phase d+2 (last used in phase d-2) */
    if (gtid == 0) ctl->work[(d + 2) & 3] = 0u;
    bool next_ready = false;

    /* this phase's work: up to two expansions, then bottom-up tiles */
    ExpandTask A = {EX_NONE, 0, Qc, bm_prev, {1, 1, 0}, true};
    ExpandTask B = {EX_NONE, 0, Qc, bm_prev, {1, 1, 0}, true};
    if (dir == DIR_TD) {
      ++td;
      if (!want_sigma) {
        A.kind = EX_DISC;
      } else if (sig_ready) { /* parents final: counts ride on the push */
        A.kind = EX_DISC_PUSH_NEW;
        next_ready = true;
      } else if (p.symmetric) { /* finish sigma(F_d) on the same list reads */
        A.kind = EX_DISC_PULL;
      } else { /* sigma(F_d) from F_{d-1}'s out-lists, discovery from F_d */
        A = {EX_PUSH_AT, d, Qp, bm_cur, {1, 1, 0}, true};
        B.kind = EX_DISC;
      }
    } else {
      ++bu;
      if (want_sigma && !sig_ready) { /* sigma(F_d): pull unless push reads far less */
        if (p.symmetric && (float)qe <= p.pull_ratio * (float)prev_qe)
          A.kind = EX_PULL;
        else
          A = {EX_PUSH_AT, d, Qp, bm_cur, {1, 1, 0}, true};
      }
    }
    const unsigned max_ept =
        p.max_ept > 0 && p.max_ept < kEPT ? (unsigned)p.max_ept : (unsigned)kEPT;
    if (TBFS_RED_PUSH && want_sigma) {
      const int nb_next = sig_bits + p.deg_bits; /* bound of F_{d+1} */
      if (A.kind == EX_DISC_PUSH_NEW)
        A.chk = !ovf_seen && !(p.deg_bits > 0 && nb_next <= 63);
      if (A.kind == EX_PUSH_AT) A.chk = !ovf_seen && !(p.deg_bits > 0 && sig_bits <= 63);
    }
    /* a small top-down level of a graph with short lists: items of
     * kShortEntries queue entries each, no owner search (expand_chunk) and
     * no edge-chunk plan */
    const bool short_level = SHORT && B.kind == EX_NONE &&
                             (A.kind == EX_DISC || A.kind == EX_DISC_PUSH_NEW) &&
                             qn <= kShortEntries * nwarps;
    if (!short_level) {
      if (A.kind != EX_NONE) A.pl = plan_expand(A.Q.qe, nwarps, max_ept);
      if (B.kind != EX_NONE) B.pl = plan_expand(B.Q.qe, nwarps, max_ept);
    }
    const unsigned n_tiles = dir == DIR_BU ? (nwords + kBuWords - 1) / kBuWords : 0u;
    const unsigned n_a = short_level ? 0u : A.pl.nch;
    const unsigned n_ab = n_a + B.pl.nch, n_all = n_ab + n_tiles;
    unsigned *wctr = &ctl->work[d & 3];
    const int lane = threadIdx.x & 31;
    /* work items: the first statically (one per warp), the rest from the
     * level's counter past the static range, so that a small level costs
     * no same-address atomics.  Static items go round-robin over the CTAs
     * (item i to CTA i % grid), so that a small level's work spreads over
     * as many SMs as it has items instead of filling the first CTAs' warps */
    unsigned item = TBFS_SPREAD_ITEMS ? (threadIdx.x >> 5) * gridDim.x + blockIdx.x
                                      : blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (short_level) {
      const unsigned first = item * kShortEntries;
      if (first < qn) run_short_item(p, d, A, first, max_ept, nx, bm_next, win, ovf);
    }
    while (item < n_all) {
      if (item < n_a) run_expand_item(p, d, A, item, nx, bm_next, win, ovf);
      else if (item < n_ab) run_expand_item(p, d, B, item - n_a, nx, bm_next, win, ovf);
      else bu_tile(p, d, nx, bm_cur, bm_next, item - n_ab);
      if (n_all <= nwarps) break;
      unsigned nxt = 0;
      if (lane == 0) nxt = nwarps + atomicAdd(wctr, 1u);
      item = __shfl_sync(FULL, nxt, 0);
    }
    prev_qn = qn;
    prev_qe = qe;
    /* test hook: CTA 0 leaves without arriving; the others' waits expire */
    if (p.inject_barrier_skip > 0 && blockIdx.x == 0 && d == p.inject_barrier_skip - 1) return;
    if (TBFS_RED_PUSH && want_sigma) { /* overflow recorded now: seen by every CTA after the barrier */
      const bool any_ovf = __any_sync(FULL, ovf);
      if (any_ovf && (threadIdx.x & 31) == 0) atomicOr(&ctl->sigma_overflow, 1);
    }
    if (!grid_barrier(ctl, p.timeout_ns, d)) break;
    sig_ready = next_ready;
    sig_bits = sig_bits + p.deg_bits < 64 ? sig_bits + p.deg_bits : 64;
    ++d;
  }
  if (__any_sync(FULL, ovf) && (threadIdx.x & 31) == 0) atomicOr(&ctl->sigma_overflow, 1);
  /* results are final after the last barrier: scatter them into the
   * caller's numbering (coalesced reads, stores need no round trip) */
  if (done && p.perm) {
    for (unsigned i = gtid; i < (unsigned)p.n; i += nthreads) {
      const int o = __ldg(p.perm + i);
      p.S_out[o] = p.S[i];
      if (want_sigma) p.sigma_out[o] = p.sigma[i];
    }
  }
  if (gtid == 0) {
    ctl->levels = d;
    ctl->td_levels = td;
    ctl->bu_levels = bu;
    ctl->visited = visited;
    ctl->edges = edges;
    if (p.trace) {
      const int slot = d < p.trace_cap - 1 ? d : p.trace_cap - 1;
      long long *rec = p.trace + 4 * (long long)slot;
      rec[0] = (long long)global_ns();
      rec[1] = 0;
      rec[2] = 0;
      rec[3] = -1;
    }
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
  /* the kernel needs ~20 KB of shared memory per CTA: carve out just enough
   * for TBFS_MIN_BLOCKS CTAs and leave the rest of the unified L1/shared
   * array to L1, which caches the depth/path-count gathers */
  int smem_sm = 0;
  e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
  if (e != cudaSuccess) return e;
  /* both instances (with and without the short-list levels) have the same
   * shared memory and register bound; the launch takes the smaller fit */
  per = 1 << 30;
  for (const void *fn : {reinterpret_cast<const void *>(bfs_persistent_kernel<false>),
                         reinterpret_cast<const void *>(bfs_persistent_kernel<true>)}) {
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, fn);
    if (e != cudaSuccess) return e;
    const size_t need = (size_t)TBFS_MIN_BLOCKS * (fa.sharedSizeBytes + 1024);
    int carve = (int)((100 * need + (size_t)smem_sm - 1) / (size_t)smem_sm);
    carve = carve < 100 ? carve : 100;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carve);
    if (e != cudaSuccess) return e;
    int fit = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, kBlock, 0);
    if (e != cudaSuccess) return e;
    per = fit < per ? fit : per;
  }
  if (per < 1) return cudaErrorInvalidConfiguration;
  out->block = kBlock;
  out->grid = sms * per;
  out->sms = sms;
  out->per_sm = per;
  return cudaSuccess;
}

cudaError_t bfs_launch(const BfsParams &p, const LaunchGeom &g, cudaStream_t s) {
  /* fewer CTAs per SM than fit when the caller's options ask for it; by
   * default 2 on short-list graphs, whose levels are many and small, so that
   * fewer CTAs meet at each barrier (2048^2 grid 13.6 vs 15.6 ms per BFS,
   * 8192^2 grid 68.4 vs 75.7, 200^3 grid 4.92 vs 5.03) */
  const int want = p.ctas_per_sm > 0 ? p.ctas_per_sm
                                     : (TBFS_SHORT_LEVELS && p.short_lists ? 2 : 0);
  const int grid = want > 0 && want < g.per_sm ? g.sms * want : g.grid;
  void *args[] = {const_cast<BfsParams *>(&p)};
  /* graphs with short out-lists run the instance with entry-aligned small
   * levels; the others run the one compiled without them */
  const void *fn = TBFS_SHORT_LEVELS && p.short_lists
                       ? reinterpret_cast<const void *>(bfs_persistent_kernel<true>)
                       : reinterpret_cast<const void *>(bfs_persistent_kernel<false>);
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(g.block), args, 0, s);
}

}  // namespace tbfs
