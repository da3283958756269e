/*
 * multi_engine.cu -- many independent traversals, each (graph, root) its own
 * instance, advancing together in one persistent cooperative launch: one
 * grid barrier per level for all of them.  Instances may live on different
 * graphs (a packed arena of many small graphs, or separately resident
 * graphs of a server) and start at different times: every instance keeps its
 * own level counter, queues and statistics in its descriptor, so a launch can
 * stop after a number of levels and a later launch can carry on with new
 * instances admitted beside the unfinished ones (continuous batching).
 *
 * Per level and instance the step is the reference's top-down semiring
 * iteration (TurboBFS_CSC_TD/bfsgputdcsc_sc.cu:159-208: f_t = A^T f over the
 * frontier, sigma += f, S = d), done as a push over the out-edges of the
 * instance's frontier queue:
 *   - an edge u -> v with S[v] == -1 claims v with atomicCAS(S[v], -1, d+1)
 *     and appends it to the next queue;
 *   - every edge that lands on a vertex at depth d+1 (claimed now, by this
 *     edge or another) adds sigma[u] to sigma[v] with a 64-bit atomicAdd;
 *     sigma[u] is final because u was claimed a level earlier.
 * Work is edge-balanced across all instances: each CTA computes the same
 * prefix of per-instance work items (rounds of 128 consecutive frontier
 * out-edges, 4 per lane, with fewer rounds per item on small levels) in
 * shared memory; a warp takes its first item by its global index and later
 * ones from a counter, locates the instance by binary search in the prefix,
 * and the owner of each edge by a 32-ary search over the instance's
 * out-degree prefix (first round) followed by a shuffle search in a window
 * of 64 queue entries.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

using dev::FULL;
using dev::grid_barrier;

#ifndef TBFS_MULTI_PER_SM
#define TBFS_MULTI_PER_SM 3
#endif

constexpr int kBlock = 256;
constexpr int kEPT = 4;                   /* consecutive edges per lane per round */
constexpr unsigned kRoundEdges = 32 * kEPT;
constexpr int kMaxRounds = 8;             /* rounds per item, fewer on small levels */

/* Append, for every lane and every bit j of take, (v[j], out-degree dg[j])
 * to a queue: one 64-bit atomic per warp reserves (count << 32 | edge sum),
 * so e[] stays the exclusive prefix of out-degrees in queue order.  All 32
 * lanes call. */
template <int N>
__device__ __forceinline__ void enqueue_n(unsigned take, const int (&v)[N], const unsigned (&dg)[N],
                                          int *q, unsigned *e, unsigned long long *ctr) {
  const int lane = threadIdx.x & 31;
  if (!__any_sync(FULL, take != 0u)) return;
  const unsigned cnt = __popc(take);
  unsigned dsum = 0;
#pragma unroll
  for (int j = 0; j < N; ++j)
    if ((take >> j) & 1u) dsum += dg[j];
  unsigned ic = cnt, id = dsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned tc = __shfl_up_sync(FULL, ic, o);
    const unsigned td = __shfl_up_sync(FULL, id, o);
    if (lane >= o) {
      ic += tc;
      id += td;
    }
  }
  const unsigned tot_c = __shfl_sync(FULL, ic, 31), tot_d = __shfl_sync(FULL, id, 31);
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(ctr, ((unsigned long long)tot_c << 32) | tot_d);
  base = __shfl_sync(FULL, base, 0);
  unsigned pos = (unsigned)(base >> 32) + ic - cnt;
  unsigned eo = (unsigned)base + id - dsum;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    if ((take >> j) & 1u) {
      q[pos] = v[j];
      e[pos] = eo;
      ++pos;
      eo += dg[j];
    }
  }
}

/* largest o < cnt with e[o] <= t, per lane (fallback of the window search) */
__device__ __forceinline__ unsigned lane_owner(const unsigned *e, unsigned cnt, unsigned t) {
  unsigned lo = 0, hi = cnt;
  while (hi - lo > 1) {
    const unsigned mid = (lo + hi) >> 1;
    if (__ldcg(e + mid) <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kBlock, TBFS_MULTI_PER_SM) multi_bfs_kernel(const MultiParams P) {
  constexpr int kWarps = kBlock / 32;
  __shared__ unsigned s_pre[kMultiMaxSlots + 1]; /* item prefix over slots      */
  __shared__ int s_d[kMultiMaxSlots];            /* level each slot runs next   */
  __shared__ unsigned s_qn[kMultiMaxSlots], s_qe[kMultiMaxSlots];
  __shared__ unsigned long long s_wsum[kWarps];  /* per-warp edge sums          */
  __shared__ int s_wact[kWarps];
  __shared__ unsigned s_wscan[kWarps];           /* per-warp item sums          */
  InstDesc *I = P.inst;
  const int ns = P.nslots;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const long long tid = (long long)blockIdx.x * kBlock + t;
  MultiCtl *ctl = P.ctl;

  for (int i = t; i < ns; i += kBlock) s_d[i] = __ldcg(&I[i].d);
  __syncthreads();

  unsigned ph = 0;
  for (; ph < (unsigned)P.max_phases; ++ph) {
    /* the host's "request waiting" flag (mapped host memory, a slow read):
     * issued now, used at the end of the level */
    int wake_now = 0;
    if (tid == 0 && P.wake) wake_now = *P.wake;
    /* ---- plan: identical in every CTA (reads counters finished before the
     * last barrier); block sums and scans by warp shuffles ---- */
    constexpr int kPer = (kMultiMaxSlots + kBlock - 1) / kBlock;
    /* every read of the plan in one round trip: the previous level's stop
     * word, each slot's done flag and queue counter, and (CTA 0) the totals
     * its bookkeeping adds to */
    const bool stop_prev = ph > 0 && __ldcg(&ctl->stop[(ph - 1) & 1u]) != 0;
    unsigned long long qvs[kPer];
    long long vis[kPer], edg[kPer];
    bool dns[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = t * kPer + j;
      qvs[j] = 0ull;
      vis[j] = edg[j] = 0;
      dns[j] = true;
      if (i < ns) {
        dns[j] = __ldcg(&I[i].done) != 0;
        qvs[j] = __ldcg(&I[i].ctr[s_d[i] % 3]);
        if (blockIdx.x == 0) {
          vis[j] = I[i].visited;
          edg[j] = I[i].edges;
        }
      }
    }
    /* a stop requested during the previous level ends the launch before
     * any bookkeeping of this one */
    if (stop_prev) break;
    unsigned qes[kPer];
    unsigned long long esum = 0;
    int act = 0, fin = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = t * kPer + j;
      qes[j] = 0;
      if (i < ns) {
        const int d = s_d[i];
        const bool done = dns[j];
        const unsigned long long qv = done ? 0ull : qvs[j];
        const unsigned qn = (unsigned)(qv >> 32), qe = (unsigned)qv;
        s_qn[i] = qn;
        s_qe[i] = qe;
        if (qn) {
          act = 1;
          qes[j] = qe;
          esum += qe;
        }
        /* bookkeeping of the instance, by CTA 0 */
        if (blockIdx.x == 0 && !done) {
          if (qn) {
            I[i].ctr[(d + 2) % 3] = 0ull;
            I[i].levels = d + 1;
            I[i].visited = vis[j] + qn;
            I[i].edges = edg[j] + qe;
          } else {
            I[i].done = 1;
            fin = 1;
          }
        }
      }
    }
    if (fin && P.stop_on_done) ctl->stop[ph & 1u] = 1; /* CTA 0 only; read after the barrier */
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(FULL, esum, o);
    const int wact = __any_sync(FULL, act);
    if (lane == 0) {
      s_wsum[wid] = esum;
      s_wact[wid] = wact;
    }
    __syncthreads();
    unsigned long long etot = 0;
    int any_act = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      etot += s_wsum[w];
      any_act |= s_wact[w];
    }
    if (!any_act) break;
    /* rounds per item: enough items for every warp on small levels */
    const unsigned nwarps = gridDim.x * kWarps;
    const unsigned long long per_warp =
        min(etot, 0xffffffffull) / ((unsigned long long)kRoundEdges * nwarps);
    const unsigned rounds = (unsigned)max(1ull, min((unsigned long long)kMaxRounds, per_warp));
    const unsigned iedges = kRoundEdges * rounds;
    unsigned items[kPer];
    unsigned sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      items[j] = (qes[j] + iedges - 1) / iedges;
      sum += items[j];
    }
    /* exclusive scan of the per-thread sums: within the warp by shuffles,
     * across the warps from their totals */
    unsigned inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned x = __shfl_up_sync(FULL, inc, o);
      if (lane >= o) inc += x;
    }
    if (lane == 31) s_wscan[wid] = inc;
    __syncthreads();
    unsigned wbase = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      const unsigned v = s_wscan[w];
      if (w < wid) wbase += v;
      total += v;
    }
    unsigned run = wbase + inc - sum;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = t * kPer + j;
      if (i < ns) s_pre[i] = run;
      run += items[j];
    }
    if (t == 0) s_pre[ns] = total;
    __syncthreads();
    if (tid == 0) ctl->work[(ph + 2) & 3u] = 0u;

    /* ---- claim items: the first one statically (global warp index), the
     * rest from the phase's counter, so that a level with few items costs
     * no same-address atomics ---- */
    unsigned it = (unsigned)wid * gridDim.x + blockIdx.x; /* round-robin over the CTAs */
    for (;; ) {
      if (it >= total) break;
      /* slot of the item: largest i with s_pre[i] <= it */
      unsigned lo = 0, hi = (unsigned)ns;
      while (hi - lo > 1) {
        const unsigned mid = (lo + hi) >> 1;
        if (s_pre[mid] <= it)
          lo = mid;
        else
          hi = mid;
      }
      const int i = (int)lo;
      InstDesc &D = I[i];
      const int d = s_d[i];
      const unsigned qn = s_qn[i], qe = s_qe[i];
      const int *q = D.q[d % 3];
      const unsigned *e = D.e[d % 3];
      int *qn_q = D.q[(d + 1) % 3];
      unsigned *qn_e = D.e[(d + 1) % 3];
      unsigned long long *ctr1 = &D.ctr[(d + 1) % 3];
      const int *rp = D.rp, *jr = D.jr;
      int *S = D.S;
      unsigned long long *sig = D.sig;
      /* counts of level d+1 have at most 1 + (d+1) deg_bits bits: below 64
       * they cannot overflow, and neither need be checked once the
       * instance's overflow is recorded; such adds are reductions whose old
       * value nobody waits for */
      const bool chk = sig && !(D.deg_bits > 0 && 1 + (long long)(d + 1) * D.deg_bits <= 63) &&
                       __ldcg(&D.ovf) == 0;
      const unsigned t0 = (it - s_pre[i]) * iedges;
      bool ovf = false;
      unsigned o0 = 0xffffffffu; /* owner of the round's first edge, once known */
      for (unsigned r = 0; r < rounds; ++r) {
        const unsigned tb = t0 + r * kRoundEdges;
        if (tb >= qe) break;
        /* owners: a 32-ary search for the item's first edge, afterwards the
         * owner of the previous round's last edge; a window of 32 queue
         * entries from there is searched with shuffles, edges beyond it
         * (runs of empty lists) by a binary search of their own */
        if (o0 == 0xffffffffu) o0 = dev::warp_find_owner(reinterpret_cast<const int *>(e), qn, tb);
        /* the window's queue entries come with their prefixes; their list
         * starts and path counts follow in one more round trip, so that an
         * edge inside the window needs only its list entry */
        const unsigned wi = o0 + lane;
        const bool in0 = wi < qn, in1 = wi + 32 < qn;
        const unsigned ew0 = in0 ? __ldcg(e + wi) : 0xffffffffu;
        const unsigned ew1 = in1 ? __ldcg(e + wi + 32) : 0xffffffffu;
        const int qw0 = in0 ? __ldcg(q + wi) : 0;
        const int qw1 = in1 ? __ldcg(q + wi + 32) : 0;
        const unsigned eend = o0 + 64 < qn ? __ldcg(e + o0 + 64) : 0xffffffffu;
        const int aw0 = in0 ? __ldg(rp + qw0) : 0;
        const int aw1 = in1 ? __ldg(rp + qw1) : 0;
        unsigned long long gw0 = 0ull, gw1 = 0ull;
        if (sig) {
          gw0 = in0 ? sig[qw0] : 0ull;
          gw1 = in1 ? sig[qw1] : 0ull;
        }
        unsigned tk[kEPT], off[kEPT], ow[kEPT];
        int u[kEPT], a[kEPT];
        unsigned long long su[kEPT];
#pragma unroll
        for (int k = 0; k < kEPT; ++k) {
          tk[k] = tb + kEPT * lane + k;
          unsigned j = 0; /* largest window index with e <= tk */
#pragma unroll
          for (int s = 32; s > 0; s >>= 1) {
            const unsigned c = j + s;
            const unsigned a0 = __shfl_sync(FULL, ew0, (int)(c & 31));
            const unsigned a1 = __shfl_sync(FULL, ew1, (int)(c & 31));
            if (c < 64 && (c < 32 ? a0 : a1) <= tk[k]) j = c;
          }
          const int src = (int)(j & 31);
          const bool hi = j >= 32;
          const unsigned b0 = __shfl_sync(FULL, ew0, src), b1 = __shfl_sync(FULL, ew1, src);
          const int u0 = __shfl_sync(FULL, qw0, src), u1 = __shfl_sync(FULL, qw1, src);
          const int c0 = __shfl_sync(FULL, aw0, src), c1 = __shfl_sync(FULL, aw1, src);
          const unsigned long long g0 = __shfl_sync(FULL, gw0, src);
          const unsigned long long g1 = __shfl_sync(FULL, gw1, src);
          ow[k] = o0 + j;
          off[k] = tk[k] - (hi ? b1 : b0);
          u[k] = hi ? u1 : u0;
          a[k] = hi ? c1 : c0;
          su[k] = hi ? g1 : g0;
          if (tk[k] < qe && tk[k] >= eend) { /* past the window: owner of its own */
            const unsigned oo = lane_owner(e, qn, tk[k]);
            ow[k] = oo;
            off[k] = tk[k] - __ldcg(e + oo);
            u[k] = __ldcg(q + oo);
            a[k] = __ldg(rp + u[k]);
            su[k] = sig ? sig[u[k]] : 0ull;
          }
        }
        int v[kEPT], sv[kEPT];
        unsigned dgo[kEPT];
#pragma unroll
        for (int k = 0; k < kEPT; ++k) v[k] = tk[k] < qe ? __ldg(jr + a[k] + (int)off[k]) : 0;
#pragma unroll
        for (int k = 0; k < kEPT; ++k) sv[k] = tk[k] < qe ? S[v[k]] : 0;
        /* degrees of the unvisited targets, in flight with the claims */
        int r0[kEPT], r1[kEPT];
#pragma unroll
        for (int k = 0; k < kEPT; ++k) {
          r0[k] = 0;
          r1[k] = 0;
          if (tk[k] < qe && sv[k] == -1) {
            r0[k] = __ldg(rp + v[k]);
            r1[k] = __ldg(rp + v[k] + 1);
          }
        }
        unsigned take = 0;
#pragma unroll
        for (int k = 0; k < kEPT; ++k) {
          if (tk[k] < qe && sv[k] == -1) {
            sv[k] = atomicCAS(S + v[k], -1, d + 1);
            if (sv[k] == -1) {
              take |= 1u << k;
              sv[k] = d + 1;
            }
          }
        }
#pragma unroll
        for (int k = 0; k < kEPT; ++k) dgo[k] = ((take >> k) & 1u) ? (unsigned)(r1[k] - r0[k]) : 0u;
        if (sig) {
#pragma unroll
          for (int k = 0; k < kEPT; ++k) {
            if (tk[k] < qe && sv[k] == d + 1) {
              const unsigned long long x = su[k];
              if (chk) {
                const unsigned long long old = atomicAdd(sig + v[k], x);
                const unsigned long long s2 = old + x;
                if (s2 < old || (s2 >> 63)) ovf = true;
              } else {
                atomicAdd(sig + v[k], x); /* result unused: a reduction */
              }
            }
          }
        }
        enqueue_n<kEPT>(take, v, dgo, qn_q, qn_e, ctr1);
        o0 = __shfl_sync(FULL, ow[kEPT - 1], 31); /* owner of the round's last edge */
      }
      if (__any_sync(FULL, ovf) && lane == 0) atomicExch(&D.ovf, 1);
      if (total <= nwarps) break;
      unsigned nx = 0;
      if (lane == 0) nx = nwarps + atomicAdd(&ctl->work[ph & 3u], 1u);
      it = __shfl_sync(FULL, nx, 0);
    }
    /* a waiting request (host flag) ends the launch after this level */
    if (tid == 0 && wake_now) ctl->stop[ph & 1u] = 1;
    if (!grid_barrier(ctl, P.timeout_ns, (int)ph)) return;
    for (int i = t; i < ns; i += kBlock)
      if (s_qn[i]) s_d[i] += 1;
    __syncthreads();
  }
  /* the level each instance runs next, for the following launch */
  if (blockIdx.x == 0)
    for (int i = t; i < ns; i += kBlock) I[i].d = s_d[i];
  if (tid == 0) ctl->phases = (int)ph;
}

/* new instances: depth 0 and count 1 at the root, queue {root} */
__global__ void multi_init_kernel(InstDesc *I, const int *slots, int k) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  InstDesc &D = I[slots[j]];
  const int r = D.inv ? D.inv[D.root] : D.root;
  D.S[r] = 0;
  if (D.sig) D.sig[r] = 1ull;
  D.q[0][0] = r;
  D.e[0][0] = 0u;
  D.ctr[0] = (1ull << 32) | (unsigned)(D.rp[r + 1] - D.rp[r]);
}

/* results in the caller's numbering: out[j] = S[inv[j]] */
__global__ void multi_gather_kernel(const int *S, const unsigned long long *sig, const int *inv,
                                    int n, int *S_out, unsigned long long *sig_out) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int v = inv ? inv[j] : (int)j;
  S_out[j] = S[v];
  if (sig_out) sig_out[j] = sig[v];
}

}  // namespace

cudaError_t multi_geometry(int device, LaunchGeom *out) {
  int sms = 0, coop = 0, per = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (e != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, multi_bfs_kernel, kBlock, 0);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  /* a few CTAs per SM: enough warps to cover the latency of the pushes,
   * fewer barrier arrivals than a fully occupied grid */
  if (per > TBFS_MULTI_PER_SM) per = TBFS_MULTI_PER_SM;
  out->block = kBlock;
  out->grid = sms * per;
  return cudaSuccess;
}

cudaError_t multi_launch(const MultiParams &p, const LaunchGeom &g, cudaStream_t s) {
  void *args[] = {const_cast<MultiParams *>(&p)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(multi_bfs_kernel), dim3(g.grid),
                                     dim3(g.block), args, 0, s);
}

cudaError_t multi_init(InstDesc *inst, const int *slots, int k, cudaStream_t s) {
  if (k <= 0) return cudaSuccess;
  multi_init_kernel<<<(k + 127) / 128, 128, 0, s>>>(inst, slots, k);
  return cudaGetLastError();
}

cudaError_t multi_gather(const int *S, const unsigned long long *sig, const int *inv, int n,
                         int *S_out, unsigned long long *sig_out, cudaStream_t s) {
  multi_gather_kernel<<<(unsigned)(((long long)n + 255) / 256), 256, 0, s>>>(S, sig, inv, n, S_out,
                                                                            sig_out);
  return cudaGetLastError();
}

}  // namespace tbfs
