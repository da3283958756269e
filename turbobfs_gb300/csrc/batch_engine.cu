/*
 * batch_engine.cu -- frontier-matrix BFS: up to 256 roots on one graph
 * advance level by level together in one persistent, cooperatively launched
 * kernel, sharing every list read among the roots.
 *
 * The reference runs one root per call (TurboBFS_CSC_TD/bfsgputdcsc_sc.cu:
 * 47-149 and its siblings); a caller with many roots -- the forward phase of
 * betweenness centrality, which is what S and sigma are for -- pays a full
 * traversal per root.  Here the roots are the columns of a frontier matrix:
 * every vertex holds a row of W 32-bit words, bit r standing for root r.
 *
 *   seen[v]   roots that have reached v
 *   F_d[v]    roots for which v is at depth d  (three rotating buffers)
 *   S_int[v][r], sig_int[v][r]   depth and path count of v from root r,
 *             written once, when r reaches v (rows of 32 W entries)
 *
 * Level d builds F_{d+1} = (OR of F_d over in-neighbours) & ~seen and, for
 * every root r newly at v, sigma_r[v] = sum of sigma_r[u] over in-neighbours
 * u with r in F_d[u] -- the same semiring step as the single-source engine,
 * one bit-column per root.  Two schedules:
 *
 *   pull  every vertex not yet reached by all roots scans its in-list.  The
 *         lanes of a vertex group (4 W lanes, lane l owning the 8 roots of
 *         row byte l) each test one in-neighbour's frontier row against the
 *         vertex's unseen mask; only rows that hit are staged in shared
 *         memory, after which every lane adds the path counts of its own
 *         roots from that neighbour's row (16-byte loads of the roots set).
 *         A vertex with more than seg_len in-list entries (a hub) is split
 *         into segments scanned by different groups; they combine with
 *         atomicOr / atomicAdd and the last segment to arrive finishes the
 *         vertex (fence + arrival counter).
 *   push  for small frontiers: edge-balanced over the out-lists of the
 *         queue of F_d, atomicOr of the new bits into F_{d+1}[v] (first
 *         touch of v appends it to the next queue), then a pull of the path
 *         counts over the in-lists of the new queue only.
 *
 * Direction rule per level: push while the frontier queue's out-edges times
 * alpha are below what a pull level costs -- the in-list entries of vertices
 * not yet reached by every root plus kVCost per vertex, since a pull visits
 * every vertex's seen row (Beamer, Asanovic, Patterson, SC 2012, with the
 * batch's unexplored edges).  Without the vertex term a pull would follow a
 * tail level of a few thousand vertices, at the cost of a pass over n.
 *
 * Path counts are exact in uint64; a sum reaching 2^63 sets the root's bit
 * in ctl->ovf.  The fast path ORs the high words of the running sums; only
 * when that shows a sum at or above 2^63 is the list rescanned with per-root
 * checks, so that the flag names exactly the roots that overflowed.
 *
 * Memory model as in the single-source engine: rows and counts read with
 * plain loads were all written before the last grid barrier; a hub's last
 * segment reads the atomically combined row with ld.global.cg after a fence.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

using dev::FULL;
using dev::grid_barrier;

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
constexpr int kPushRounds = 8;    /* 32-edge rounds per push work item         */
constexpr int kClear = 256;       /* queue entries per row-clearing item        */
constexpr int kVCost = 4;         /* a vertex costs like this many list entries */
#ifndef TBFS_BATCH_ITEM
#define TBFS_BATCH_ITEM 512
#endif
constexpr long long kItemCost = TBFS_BATCH_ITEM; /* list entries + vertex costs per item */
#ifndef TBFS_BATCH_HITS
#define TBFS_BATCH_HITS 3
#endif
constexpr int kHitBatch = TBFS_BATCH_HITS; /* hit rows whose counts are fetched per round trip */
constexpr int kStageU64 = kHitBatch * 32 * 8; /* per-warp stage: hits x lanes x 8 counts */

/* ---- row access ---------------------------------------------------------- */

template <int W>
__device__ __forceinline__ void load_row(const unsigned *p, unsigned (&r)[W]) {
  if constexpr (W == 8) {
    const uint4 a = *reinterpret_cast<const uint4 *>(p);
    const uint4 b = *reinterpret_cast<const uint4 *>(p + 4);
    r[0] = a.x, r[1] = a.y, r[2] = a.z, r[3] = a.w, r[4] = b.x, r[5] = b.y, r[6] = b.z, r[7] = b.w;
  } else if constexpr (W == 4) {
    const uint4 a = *reinterpret_cast<const uint4 *>(p);
    r[0] = a.x, r[1] = a.y, r[2] = a.z, r[3] = a.w;
  } else if constexpr (W == 2) {
    const uint2 a = *reinterpret_cast<const uint2 *>(p);
    r[0] = a.x, r[1] = a.y;
  } else {
    r[0] = *p;
  }
}

/* the same through L2 (rows combined by atomics during the current phase) */
template <int W>
__device__ __forceinline__ void load_row_cg(const unsigned *p, unsigned (&r)[W]) {
  if constexpr (W == 8) {
    const uint4 a = __ldcg(reinterpret_cast<const uint4 *>(p));
    const uint4 b = __ldcg(reinterpret_cast<const uint4 *>(p + 4));
    r[0] = a.x, r[1] = a.y, r[2] = a.z, r[3] = a.w, r[4] = b.x, r[5] = b.y, r[6] = b.z, r[7] = b.w;
  } else if constexpr (W == 4) {
    const uint4 a = __ldcg(reinterpret_cast<const uint4 *>(p));
    r[0] = a.x, r[1] = a.y, r[2] = a.z, r[3] = a.w;
  } else if constexpr (W == 2) {
    const uint2 a = __ldcg(reinterpret_cast<const uint2 *>(p));
    r[0] = a.x, r[1] = a.y;
  } else {
    r[0] = __ldcg(p);
  }
}

template <int W>
__device__ __forceinline__ void store_row(unsigned *p, const unsigned (&r)[W]) {
  if constexpr (W == 8) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(r[0], r[1], r[2], r[3]);
    *reinterpret_cast<uint4 *>(p + 4) = make_uint4(r[4], r[5], r[6], r[7]);
  } else if constexpr (W == 4) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(r[0], r[1], r[2], r[3]);
  } else if constexpr (W == 2) {
    *reinterpret_cast<uint2 *>(p) = make_uint2(r[0], r[1]);
  } else {
    *p = r[0];
  }
}

/* a[i] for a run-time i without dynamic register indexing */
template <int W>
__device__ __forceinline__ unsigned pick(const unsigned (&a)[W], int i) {
  unsigned x = a[0];
#pragma unroll
  for (int w = 1; w < W; ++w)
    if (i == w) x = a[w];
  return x;
}

/* Lanes of one vertex group: G = 4 W lanes for the 32 W roots of a row.
 * Lane gl owns the root pairs c_q = gl + G q (q = 0..3), i.e. roots 2 c_q
 * and 2 c_q + 1.  A pair is one 16-byte chunk of a path-count row, so the
 * chunks of the G lanes for one q are contiguous: copies and stores of a
 * group are coalesced, and each lane's staged chunks are conflict-free.
 * Frontier rows store root r = 2 c_q + t at bit position 8 gl + 2 q + t
 * (bit_of_root), so a lane's 8 roots are exactly byte gl of every row. */
template <int W>
struct Grp {
  static constexpr int G = 4 * W;
  static constexpr int PER_WARP = 32 / G;
  int lane, gid, gl, gbase;
  unsigned gmask;
  __device__ __forceinline__ Grp() {
    lane = threadIdx.x & 31;
    gid = lane / G;
    gl = lane % G;
    gbase = gid * G;
    gmask = G == 32 ? FULL : (((1u << G) - 1u) << gbase);
  }
  /* root of bit b of this lane's mask */
  __device__ __forceinline__ int root(int b) const { return 2 * (gl + G * (b >> 1)) + (b & 1); }
};

/* bit position of root r in a frontier row of W words (see Grp) */
__device__ __host__ __forceinline__ int bit_of_root(int r, int W) {
  const int c = r >> 1, G = 4 * W;
  return 8 * (c % G) + 2 * (c / G) + (r & 1);
}

/* this lane's 8-bit mask (its byte) of a row held in registers */
template <int W>
__device__ __forceinline__ unsigned lane_bits(const unsigned (&row)[W], const Grp<W> &g) {
  return (pick<W>(row, g.gl >> 2) >> (8 * (g.gl & 3))) & 0xffu;
}

/* the same for a row in shared memory */
template <int W>
__device__ __forceinline__ unsigned lane_bits_smem(const unsigned *row, const Grp<W> &g) {
  return reinterpret_cast<const unsigned char *>(row)[g.gl]; /* byte gl: words are little-endian */
}

template <int W>
__device__ __forceinline__ void group_or(unsigned (&x)[W], unsigned gmask) {
#pragma unroll
  for (int o = 1; o < 4 * W; o <<= 1)
#pragma unroll
    for (int w = 0; w < W; ++w) x[w] |= __shfl_xor_sync(gmask, x[w], o);
}

/* found as left by scan_list -> the group's found row in every lane */
template <int W, int SIG>
__device__ __forceinline__ void finish_found(unsigned (&found)[W], const Grp<W> &g) {
  if constexpr (SIG != 0) {
    /* word w holds the bytes of lanes 4w .. 4w+3 */
    const unsigned b = found[0];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      unsigned x = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) x |= __shfl_sync(g.gmask, b, g.gbase + 4 * w + k) << (8 * k);
      found[w] = x;
    }
  } else {
    group_or<W>(found, g.gmask);
  }
}

/* Per-warp shared memory: m (32 x W words) stages the hit rows' masks;
 * stage (kHitBatch x 4 x 32 lanes x 2 counts) receives the 16-byte chunks of
 * path counts each lane fetches asynchronously for its own roots: chunk q of
 * hit b of a lane at stage[((4 b + q) * 32 + lane) * 2]. */
struct WarpSmem {
  unsigned *m;
  unsigned long long *stage;
};

/* cp.async of 16 bytes from g + GOFF to shared address s + SOFF when pred is
 * nonzero: predicated, offsets as immediates */
template <int SOFF, int GOFF>
__device__ __forceinline__ void cp_async16_off(unsigned s, const void *g, unsigned pred) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\t"
      "@p cp.async.cg.shared.global [%0+%3], [%1+%4], 16;\n\t}" ::"r"(s),
      "l"(g), "r"(pred), "n"(SOFF), "n"(GOFF)
      : "memory");
}

/* cp.async of 8 bytes (through L1) */
template <int SOFF, int GOFF>
__device__ __forceinline__ void cp_async8_off(unsigned s, const void *g, unsigned pred) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\t"
      "@p cp.async.ca.shared.global [%0+%3], [%1+%4], 8;\n\t}" ::"r"(s),
      "l"(g), "r"(pred), "n"(SOFF), "n"(GOFF)
      : "memory");
}

/* the four root-pair chunks of one hit row for a lane of a G-lane group.
 * 64-bit counts: chunk q (16 bytes) from g + 16 G q bytes into shared
 * s + 512 q bytes; 32-bit counts (NR): chunk q (8 bytes) from g + 8 G q
 * bytes into s + 256 q bytes; each copied if pair q of the lane's byte lm is
 * set */
template <int G, bool NR>
__device__ __forceinline__ void fetch_pairs(unsigned s, const void *g, unsigned lm) {
  if constexpr (NR) {
    cp_async8_off<0, 0>(s, g, lm & 0x03u);
    cp_async8_off<256, 8 * G>(s, g, lm & 0x0cu);
    cp_async8_off<512, 16 * G>(s, g, lm & 0x30u);
    cp_async8_off<768, 24 * G>(s, g, lm & 0xc0u);
  } else {
    cp_async16_off<0, 0>(s, g, lm & 0x03u);
    cp_async16_off<512, 16 * G>(s, g, lm & 0x0cu);
    cp_async16_off<1024, 32 * G>(s, g, lm & 0x30u);
    cp_async16_off<1536, 48 * G>(s, g, lm & 0xc0u);
  }
}

/* wait for this thread's outstanding cp.async copies */
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

/* ---- path-count accumulation ---------------------------------------------- */

template <bool EXACT>
__device__ __forceinline__ void add1(unsigned long long &a, unsigned long long x, unsigned lm,
                                     int b, unsigned &ovh, unsigned &ovm) {
  if ((lm >> b) & 1u) {
    a += x;
    if (EXACT) {
      if (a >> 63) ovm |= 1u << b;
    } else {
      ovh |= (unsigned)(a >> 32);
    }
  }
}

/* acc[b] += the staged count of bit b of lane mask lm (one hit).  Fast path:
 * ovh collects the high words (bit 31 set once any sum reached 2^63); EXACT:
 * ovm gets the bit of every root whose sum reached 2^63. */
template <bool EXACT, bool NR>
__device__ __forceinline__ void acc_staged(const void *slot_v, unsigned lm,
                                           unsigned long long (&acc)[8], unsigned &ovh,
                                           unsigned &ovm) {
  const unsigned long long *slot = reinterpret_cast<const unsigned long long *>(slot_v);
  if constexpr (NR) {
    /* 32-bit counts: 8-byte chunks 256 bytes apart; any high word set means
     * a count that 32 bits cannot hold (the launch is then redone wide) */
    const unsigned *s32 = reinterpret_cast<const unsigned *>(slot_v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint2 x = *reinterpret_cast<const uint2 *>(s32 + q * 64);
      if (lm & (1u << (2 * q))) acc[2 * q] += x.x;
      if (lm & (2u << (2 * q))) acc[2 * q + 1] += x.y;
      ovh |= (unsigned)(acc[2 * q] >> 32) | (unsigned)(acc[2 * q + 1] >> 32);
    }
  } else if constexpr (!EXACT) {
    /* branch-free: every chunk slot is read (a slot not copied this time
     * holds a stale value, which no add takes), the adds are predicated on
     * the root bits, and one OR per pair collects both high words */
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const ulonglong2 x = *reinterpret_cast<const ulonglong2 *>(slot + q * 64);
      if (lm & (1u << (2 * q))) acc[2 * q] += x.x;
      if (lm & (2u << (2 * q))) acc[2 * q + 1] += x.y;
      ovh |= (unsigned)(acc[2 * q] >> 32) | (unsigned)(acc[2 * q + 1] >> 32);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if ((lm >> (2 * q)) & 3u) {
        const ulonglong2 x = *reinterpret_cast<const ulonglong2 *>(slot + q * 64);
        add1<EXACT>(acc[2 * q], x.x, lm, 2 * q, ovh, ovm);
        add1<EXACT>(acc[2 * q + 1], x.y, lm, 2 * q + 1, ovh, ovm);
      }
    }
  }
}

/* record the overflow of the roots of lane mask ovm */
template <int W>
__device__ __forceinline__ void report_overflow(const BatchParams &p, unsigned ovm, const Grp<W> &g) {
  while (ovm) {
    const int b = __ffs(ovm) - 1;
    ovm &= ovm - 1u;
    const int r = g.root(b);
    atomicOr(&p.ctl->ovf[r >> 5], 1u << (r & 31));
  }
}

/* Scan in-list entries [lo, hi) of one vertex with its group: the OR of
 * F_d[u] & want over the entries is collected in found -- without SIG as
 * rows (each lane its own entries; finish_found ORs them over the group),
 * with SIG as the lane's own byte in found[0] (finish_found assembles the
 * row), which keeps seven registers free for the path counts.  With SIG,
 * every lane also adds to acc the path counts of its roots set in F_d[u] &
 * want.  sm: the warp's 32 x W staging words. */
template <int W, int SIG, bool EXACT>
__device__ __forceinline__ void scan_list(const BatchParams &p, const unsigned *Fd, int lo, int hi,
                                          const unsigned (&want)[W], unsigned (&found)[W],
                                          unsigned long long (&acc)[8], unsigned &ovh,
                                          unsigned &ovm, const WarpSmem &sm, const Grp<W> &g) {
  constexpr int G = 4 * W;
  constexpr int RS = 32 * W;
  for (int base = lo; base < hi; base += G) {
    const int i = base + g.gl;
    const bool has = i < hi;
    int u = 0;
    unsigned m[W];
    bool any = false;
    if (has) {
      u = __ldg(p.ic + i);
      load_row<W>(Fd + (size_t)u * W, m);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        m[w] &= want[w];
        any |= m[w] != 0u;
      }
    } else {
#pragma unroll
      for (int w = 0; w < W; ++w) m[w] = 0u;
    }
    if constexpr (SIG == 0) {
#pragma unroll
      for (int w = 0; w < W; ++w) found[w] |= m[w];
    }
    if (SIG) {
      unsigned hits = __ballot_sync(g.gmask, any);
      if (hits) {
        if (any) store_row<W>(sm.m + g.lane * W, m);
        __syncwarp(g.gmask);
        hits >>= g.gbase;
        /* kHitBatch hit rows per round trip: every lane copies the chunks of
         * its roots that are set (16 bytes per root pair) into its own stage
         * slots, waits for its own copies only, then accumulates */
        constexpr bool NR = SIG == 2;
        constexpr unsigned kHitBytes = NR ? 1024u : 2048u; /* stage bytes of one hit */
        unsigned char *mine = reinterpret_cast<unsigned char *>(sm.stage) + g.lane * (NR ? 8 : 16);
        const unsigned s_mine = (unsigned)__cvta_generic_to_shared(mine);
        do {
          unsigned lms[kHitBatch];
#pragma unroll
          for (int b = 0; b < kHitBatch; ++b) {
            lms[b] = 0u;
            if (hits) {
              const int j = __ffs(hits) - 1;
              hits &= hits - 1u;
              const int uj = __shfl_sync(g.gmask, u, g.gbase + j);
              const unsigned lm = lane_bits_smem<W>(sm.m + (g.gbase + j) * W, g);
              lms[b] = lm;
              found[0] |= lm;
              const void *row =
                  NR ? (const void *)(reinterpret_cast<const unsigned *>(p.sig_int) +
                                      (size_t)uj * RS + 2 * g.gl)
                     : (const void *)(p.sig_int + (size_t)uj * RS + 2 * g.gl);
              fetch_pairs<G, NR>(s_mine + kHitBytes * (unsigned)b, row, lm);
            }
          }
          cp_async_wait_all();
#pragma unroll
          for (int b = 0; b < kHitBatch; ++b)
            if (lms[b]) acc_staged<EXACT, NR>(mine + kHitBytes * b, lms[b], acc, ovh, ovm);
        } while (hits);
        __syncwarp(g.gmask);
      }
    }
  }
}

/* Per-root overflow bits of this lane's roots for the sums over [lo, hi):
 * the slow, exact rescan, run only when the fast path saw a high bit. */
template <int W>
__device__ __forceinline__ unsigned exact_overflow(const BatchParams &p, const unsigned *Fd, int lo,
                                                   int hi, const unsigned (&want)[W], const WarpSmem &sm,
                                                   const Grp<W> &g) {
  unsigned f[W];
#pragma unroll
  for (int w = 0; w < W; ++w) f[w] = 0u;
  unsigned long long a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned oh = 0, om = 0;
  scan_list<W, 1, true>(p, Fd, lo, hi, want, f, a, oh, om, sm, g);
  return om;
}

/* write depth d+1 (and the counts) of the roots of lane mask nb at vertex v */
template <int W, int SIG>
__device__ __forceinline__ void write_new(const BatchParams &p, int d, int v, unsigned nb,
                                          const unsigned long long (&acc)[8], const Grp<W> &g) {
  constexpr int RS = 32 * W;
  constexpr int G = 4 * W;
  if (!nb) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const unsigned pr = (nb >> (2 * q)) & 3u;
    if (!pr) continue;
    const size_t at = (size_t)v * RS + 2 * (g.gl + G * q);
    unsigned *c32 = reinterpret_cast<unsigned *>(p.sig_int);
    if (pr == 3u) {
      *reinterpret_cast<int2 *>(p.S_int + at) = make_int2(d + 1, d + 1);
      if (SIG == 2)
        *reinterpret_cast<uint2 *>(c32 + at) = make_uint2((unsigned)acc[2 * q], (unsigned)acc[2 * q + 1]);
      else if (SIG)
        *reinterpret_cast<ulonglong2 *>(p.sig_int + at) = make_ulonglong2(acc[2 * q], acc[2 * q + 1]);
    } else {
      const int t = pr == 2u ? 1 : 0;
      p.S_int[at + t] = d + 1;
      if (SIG == 2) c32[at + t] = (unsigned)(t ? acc[2 * q + 1] : acc[2 * q]);
      else if (SIG) p.sig_int[at + t] = t ? acc[2 * q + 1] : acc[2 * q];
    }
  }
}

template <int W>
__device__ __forceinline__ bool row_full(const BatchParams &p, const unsigned (&a)[W],
                                         const unsigned (&b)[W]) {
  bool f = true;
#pragma unroll
  for (int w = 0; w < W; ++w) f &= (a[w] | b[w]) == p.valid[w];
  return f;
}

/* ---- per-vertex work ------------------------------------------------------- */

/* pull level, whole in-list of v (not a hub): discover and count */
template <int W, int SIG>
__device__ __forceinline__ void pull_vertex(const BatchParams &p, int d, int v, int lo, int hi,
                                            const unsigned (&sn)[W], const unsigned *Fd,
                                            unsigned *F1, const WarpSmem &sm, const Grp<W> &g,
                                            bool &take, bool &full) {
  unsigned want[W], found[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    want[w] = p.valid[w] & ~sn[w];
    found[w] = 0u;
  }
  unsigned long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned ovh = 0, ovm = 0;
  scan_list<W, SIG, false>(p, Fd, lo, hi, want, found, acc, ovh, ovm, sm, g);
  bool anyf = false;
#pragma unroll
  for (int w = 0; w < W; ++w) anyf |= found[w] != 0u;
  take = false;
  full = false;
  if (!__any_sync(g.gmask, anyf)) return;
  finish_found<W, SIG>(found, g);
  if (SIG == 2) {
    if (__any_sync(g.gmask, ovh != 0u) && g.gl == 0) p.ctl->wide = 1;
  } else if (SIG && __any_sync(g.gmask, (ovh >> 31) != 0u)) {
    ovm = exact_overflow<W>(p, Fd, lo, hi, want, sm, g);
    report_overflow<W>(p, ovm, g);
  }
  write_new<W, SIG>(p, d, v, lane_bits<W>(found, g), acc, g);
  /* seen rows hold valid roots only, so sn = valid & ~want: sn need not
   * stay live across the scan */
  if (g.gl < W) {
    const unsigned fw = pick<W>(found, g.gl);
    if (fw) {
      F1[(size_t)v * W + g.gl] = fw;
      p.seen[(size_t)v * W + g.gl] = (p.valid[g.gl] & ~pick<W>(want, g.gl)) | fw;
    }
  }
  take = true;
  bool f = true;
#pragma unroll
  for (int w = 0; w < W; ++w) f &= found[w] == want[w];
  full = f;
}

/* Fold a segment's partial result into hub h: new bits into F1 (pull only),
 * partial counts into sig_int by atomics.  found must be group-reduced. */
template <int W, int SIG, bool DISC>
__device__ __forceinline__ void commit_segment(const BatchParams &p, int h, const unsigned (&found)[W],
                                               const unsigned long long (&acc)[8], unsigned ovh,
                                               const unsigned *Fd, int lo, int hi,
                                               const unsigned (&want)[W], unsigned *F1,
                                               const WarpSmem &sm, const Grp<W> &g) {
  constexpr int RS = 32 * W;
  if (DISC && g.gl < W) {
    const unsigned fw = pick<W>(found, g.gl);
    if (fw) atomicOr(&F1[(size_t)h * W + g.gl], fw);
  }
  if (SIG == 2) { /* 32-bit counts: any count past 32 bits redoes the launch wide */
    bool wide = __any_sync(g.gmask, ovh != 0u);
    const unsigned nb = lane_bits<W>(found, g);
    if (nb) {
      unsigned *crow = reinterpret_cast<unsigned *>(p.sig_int) + (size_t)h * RS;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        if ((nb >> b) & 1u) {
          const unsigned x = (unsigned)acc[b];
          const unsigned old = atomicAdd(crow + g.root(b), x);
          if (old + x < old) wide = true;
        }
      }
    }
    if (wide) p.ctl->wide = 1;
  } else if (SIG) {
    unsigned ovm = 0;
    if (__any_sync(g.gmask, (ovh >> 31) != 0u)) ovm = exact_overflow<W>(p, Fd, lo, hi, want, sm, g);
    const unsigned nb = lane_bits<W>(found, g);
    if (nb) {
      unsigned long long *crow = p.sig_int + (size_t)h * RS;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        if ((nb >> b) & 1u) {
          const unsigned long long old = atomicAdd(crow + g.root(b), acc[b]);
          const unsigned long long s = old + acc[b];
          if (s < old || (s >> 63)) ovm |= 1u << b;
        }
      }
    }
    report_overflow<W>(p, ovm, g);
  }
}

/* arrival of one segment of hub h; true on the group of the last one */
template <int W>
__device__ __forceinline__ bool arrive_last(const BatchParams &p, int h, unsigned nseg,
                                            const Grp<W> &g) {
  __threadfence();
  __syncwarp(g.gmask);
  unsigned last = 0;
  if (g.gl == 0) {
    const unsigned old = atomicAdd(&p.seg_arrive[h], 1u);
    last = ((old + 1u) % nseg) == 0u ? 1u : 0u;
  }
  last = __shfl_sync(g.gmask, last, g.gbase);
  if (last) __threadfence();
  return last != 0u;
}

/* pull level, one segment of hub h */
template <int W, int SIG>
__device__ __forceinline__ void pull_segment(const BatchParams &p, int d, int h, int lo, int hi,
                                             unsigned nseg, const unsigned (&sn)[W],
                                             const unsigned *Fd, unsigned *F1, const WarpSmem &sm,
                                             const Grp<W> &g, bool &take, bool &full) {
  unsigned want[W], found[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    want[w] = p.valid[w] & ~sn[w];
    found[w] = 0u;
  }
  unsigned long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned ovh = 0, ovm = 0;
  scan_list<W, SIG, false>(p, Fd, lo, hi, want, found, acc, ovh, ovm, sm, g);
  bool anyf = false;
#pragma unroll
  for (int w = 0; w < W; ++w) anyf |= found[w] != 0u;
  if (__any_sync(g.gmask, anyf)) {
    finish_found<W, SIG>(found, g);
    commit_segment<W, SIG, true>(p, h, found, acc, ovh, Fd, lo, hi, want, F1, sm, g);
  }
  take = false;
  full = false;
  if (!arrive_last<W>(p, h, nseg, g)) return;
  unsigned nx[W];
  load_row_cg<W>(F1 + (size_t)h * W, nx);
  bool anyn = false;
#pragma unroll
  for (int w = 0; w < W; ++w) anyn |= nx[w] != 0u;
  if (!anyn) return;
  unsigned long long none[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  write_new<W, false>(p, d, h, lane_bits<W>(nx, g), none, g);
  if (g.gl < W) {
    const unsigned fw = pick<W>(nx, g.gl);
    if (fw) p.seen[(size_t)h * W + g.gl] = (p.valid[g.gl] & ~pick<W>(want, g.gl)) | fw;
  }
  take = true;
  bool f = true;
#pragma unroll
  for (int w = 0; w < W; ++w) f &= nx[w] == want[w];
  full = f;
}

/* push level, second phase: counts of the roots new at v (all of them known
 * now in F1[v]); finishes v (depths, seen, queue-membership bit) */
template <int W, int SIG>
__device__ __forceinline__ void count_vertex(const BatchParams &p, int d, int v, int lo, int hi,
                                             const unsigned *Fd, const unsigned *F1, const WarpSmem &sm,
                                             const Grp<W> &g, bool &full) {
  unsigned want[W], sn[W];
  load_row<W>(F1 + (size_t)v * W, want);
  load_row<W>(p.seen + (size_t)v * W, sn);
  unsigned long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (SIG) {
    unsigned found[W];
#pragma unroll
    for (int w = 0; w < W; ++w) found[w] = 0u;
    unsigned ovh = 0, ovm = 0;
    scan_list<W, SIG, false>(p, Fd, lo, hi, want, found, acc, ovh, ovm, sm, g);
    if (SIG == 2) {
      if (__any_sync(g.gmask, ovh != 0u) && g.gl == 0) p.ctl->wide = 1;
    } else if (__any_sync(g.gmask, (ovh >> 31) != 0u)) {
      ovm = exact_overflow<W>(p, Fd, lo, hi, want, sm, g);
      report_overflow<W>(p, ovm, g);
    }
  }
  write_new<W, SIG>(p, d, v, lane_bits<W>(want, g), acc, g);
  if (g.gl < W) {
    const unsigned ww = pick<W>(want, g.gl);
    if (ww) p.seen[(size_t)v * W + g.gl] = pick<W>(sn, g.gl) | ww;
  }
  if (g.gl == 0) atomicAnd(&p.touched[v >> 5], ~(1u << (v & 31)));
  full = row_full<W>(p, sn, want);
}

/* push level, second phase, one segment of hub h (path counts only) */
template <int W, int SIG>
__device__ __forceinline__ void count_segment(const BatchParams &p, int d, int h, int lo, int hi,
                                              unsigned nseg, const unsigned *Fd, unsigned *F1,
                                              const WarpSmem &sm, const Grp<W> &g, bool &full) {
  unsigned want[W], found[W];
  load_row<W>(F1 + (size_t)h * W, want);
#pragma unroll
  for (int w = 0; w < W; ++w) found[w] = 0u;
  unsigned long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned ovh = 0, ovm = 0;
  scan_list<W, SIG, false>(p, Fd, lo, hi, want, found, acc, ovh, ovm, sm, g);
  bool anyf = false;
#pragma unroll
  for (int w = 0; w < W; ++w) anyf |= found[w] != 0u;
  if (__any_sync(g.gmask, anyf)) {
    finish_found<W, SIG>(found, g);
    commit_segment<W, SIG, false>(p, h, found, acc, ovh, Fd, lo, hi, want, F1, sm, g);
  }
  full = false;
  if (!arrive_last<W>(p, h, nseg, g)) return;
  unsigned sn[W];
  load_row<W>(p.seen + (size_t)h * W, sn);
  unsigned long long none[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  write_new<W, false>(p, d, h, lane_bits<W>(want, g), none, g);
  if (g.gl < W) {
    const unsigned ww = pick<W>(want, g.gl);
    if (ww) p.seen[(size_t)h * W + g.gl] = pick<W>(sn, g.gl) | ww;
  }
  if (g.gl == 0) atomicAnd(&p.touched[h >> 5], ~(1u << (h & 31)));
  full = row_full<W>(p, sn, want);
}

/* ---- queues ------------------------------------------------------------------ */

/* Append, for every lane with take set, (v, out-degree dg) to a queue: one
 * 64-bit atomic per warp reserves (count << 32 | edge sum), so e[] stays the
 * exclusive prefix of out-degrees in queue order.  All 32 lanes call. */
__device__ __forceinline__ void warp_enqueue(bool take, int v, unsigned dg, int *q, unsigned *e,
                                             unsigned long long *ctr) {
  const int lane = threadIdx.x & 31;
  const unsigned bal = __ballot_sync(FULL, take);
  if (!bal) return;
  const unsigned mine = take ? dg : 0u;
  unsigned inc = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(FULL, inc, o);
    if (lane >= o) inc += t;
  }
  const unsigned tot = __shfl_sync(FULL, inc, 31);
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(ctr, ((unsigned long long)__popc(bal) << 32) | tot);
  base = __shfl_sync(FULL, base, 0);
  if (take) {
    const unsigned pos = (unsigned)(base >> 32) + __popc(bal & ((1u << lane) - 1u));
    q[pos] = v;
    e[pos] = (unsigned)base + inc - mine;
  }
}

__device__ __forceinline__ unsigned nsegs(int deg, int seg_len) {
  return (unsigned)((deg + seg_len - 1) / seg_len);
}

/* Smallest i in [0, cnt] with f(i) >= target, f nondecreasing on [0, cnt)
 * and f(cnt) taken as +infinity; 32-ary search, all 32 lanes call with the
 * same arguments. */
template <class F>
__device__ __forceinline__ unsigned warp_lower_bound(F f, unsigned cnt, long long target) {
  const int lane = threadIdx.x & 31;
  unsigned lo = 0, hi = cnt;
  while (hi - lo > 32) {
    const unsigned step = (hi - lo + 31) / 32;
    const unsigned pidx = lo + lane * step;
    const bool pred = pidx < hi && f(pidx) < target;
    const unsigned c = __popc(__ballot_sync(FULL, pred));
    if (c == 0) return lo;
    const unsigned nhi = lo + c * step;
    lo = lo + (c - 1) * step + 1;
    hi = nhi < hi ? nhi : hi;
  }
  const unsigned pidx = lo + lane;
  const bool pred = pidx < hi && f(pidx) < target;
  return lo + __popc(__ballot_sync(FULL, pred));
}

/* largest i < cnt with pre[i] <= t (pre nondecreasing, pre[0] = 0) */
template <class T>
__device__ __forceinline__ unsigned upper_owner(const T *pre, unsigned cnt, unsigned t) {
  unsigned lo = 0, hi = cnt;
  while (hi - lo > 1) {
    const unsigned mid = (lo + hi) >> 1;
    if ((unsigned)__ldcg(pre + mid) <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

/* ---- the kernel ------------------------------------------------------------- */

#ifndef TBFS_BATCH_MINB
#define TBFS_BATCH_MINB 3 /* 3 CTAs of 256 per SM: 24 warps hide more latency than 128 registers would save */
#endif

template <int W, int SIG>
__global__ void __launch_bounds__(kBlock, TBFS_BATCH_MINB) fm_bfs_kernel(const BatchParams p) {
  constexpr int PER = Grp<W>::PER_WARP;
  constexpr int RS = 32 * W;
  __shared__ __align__(16) unsigned s_m[kWarps][32 * W];
  __shared__ int s_bv[kWarps][32];
  __shared__ unsigned s_bd[kWarps][32];
  const Grp<W> g;
  const int wid = threadIdx.x >> 5;
  extern __shared__ __align__(16) unsigned long long s_dyn[]; /* kWarps x kStageU64 with SIG */
  const WarpSmem sm{s_m[wid], SIG ? s_dyn + (size_t)wid * kStageU64 : nullptr};
  BatchCtl *ctl = p.ctl;
  const long long tid = (long long)blockIdx.x * kBlock + threadIdx.x;
  const long long nth = (long long)gridDim.x * kBlock;
  const int n = p.n;

  /* clear the rows and per-vertex words; zero the hubs' count rows (they are
   * summed into by atomics) */
  const long long rows = (long long)n * W;
  for (long long i = tid; i < rows; i += nth) {
    p.seen[i] = 0u;
    p.F[0][i] = 0u;
    p.F[1][i] = 0u;
    p.F[2][i] = 0u;
  }
  for (long long i = tid; i < ((long long)n + 31) / 32; i += nth) p.touched[i] = 0u;
  for (long long i = tid; i < n; i += nth) p.seg_arrive[i] = 0u;
  if (SIG == 2) {
    for (long long i = tid; i < (long long)p.nhub * RS; i += nth)
      reinterpret_cast<unsigned *>(p.sig_int)[(size_t)__ldg(p.hubs + i / RS) * RS + i % RS] = 0u;
  } else if (SIG) {
    for (long long i = tid; i < (long long)p.nhub * RS; i += nth)
      p.sig_int[(size_t)__ldg(p.hubs + i / RS) * RS + i % RS] = 0ull;
  }
  if (!grid_barrier(ctl, p.timeout_ns, -1)) return;

  /* roots (k <= 256 = kBlock): CTA 0 sets their bits, depth 0, count 1, and
   * builds Q_0 from the distinct root vertices */
  if (blockIdx.x == 0) {
    __shared__ int s_rv[kBlock];
    const int t = threadIdx.x;
    int v = 0;
    if (t < p.k) {
      v = __ldg(p.roots + t);
      if (p.inv) v = __ldg(p.inv + v);
      const int b = bit_of_root(t, W);
      atomicOr(&p.seen[(size_t)v * W + (b >> 5)], 1u << (b & 31));
      atomicOr(&p.F[0][(size_t)v * W + (b >> 5)], 1u << (b & 31));
      p.S_int[(size_t)v * RS + t] = 0;
      if (SIG == 2) reinterpret_cast<unsigned *>(p.sig_int)[(size_t)v * RS + t] = 1u;
      else if (SIG) p.sig_int[(size_t)v * RS + t] = 1ull;
    }
    s_rv[t] = v;
    __syncthreads();
    bool first = t < p.k;
    for (int j = 0; j < t && first; ++j)
      if (s_rv[j] == v) first = false;
    const unsigned dg = first ? (unsigned)(__ldg(p.rp + v + 1) - __ldg(p.rp + v)) : 0u;
    const unsigned one = first ? 1u : 0u;
    /* inclusive scans of the first-occurrence flags and of the degrees */
    __shared__ unsigned s_cnt[kBlock], s_deg[kBlock];
    s_cnt[t] = one;
    s_deg[t] = dg;
    __syncthreads();
    for (int o = 1; o < kBlock; o <<= 1) {
      const unsigned c = t >= o ? s_cnt[t - o] : 0u;
      const unsigned e = t >= o ? s_deg[t - o] : 0u;
      __syncthreads();
      s_cnt[t] += c;
      s_deg[t] += e;
      __syncthreads();
    }
    if (first) {
      const unsigned pos = s_cnt[t] - 1u;
      p.q[0][pos] = v;
      p.e[0][pos] = s_deg[t] - dg;
    }
    if (t == kBlock - 1) ctl->qctr[0] = ((unsigned long long)s_cnt[t] << 32) | s_deg[t];
  }
  if (!grid_barrier(ctl, p.timeout_ns, -1)) return;

  unsigned ph = 0;            /* phase counter: work slot ph % 4 */
  unsigned long long md = 0;  /* this lane's newly finished in-list entries  */
  long long m_done = 0;       /* in-list entries of vertices every root reached,
                                 summed from the per-level slots (identical in
                                 every thread, so every CTA takes the same
                                 direction) */

  /* work items of a phase: the first one statically (global warp index),
   * later ones from the phase's counter (after the static range) */
  const unsigned nwarps = gridDim.x * kWarps;
  const unsigned gwarp = blockIdx.x * kWarps + wid;
  bool first_claim = true;
  auto claim = [&](unsigned total) -> unsigned {
    if (first_claim) {
      first_claim = false;
      return gwarp;
    }
    if (total <= nwarps) return 0xffffffffu; /* the static range covered all */
    unsigned it = 0;
    if (g.lane == 0) it = nwarps + atomicAdd(&ctl->work[ph & 3u], 1u);
    return __shfl_sync(FULL, it, 0);
  };
  /* entries finished during level d go to slot (d + 1) % 4, read at the
   * start of level d + 1 */
  auto flush_md = [&](int d) {
    unsigned long long x = md;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    if (g.lane == 0 && x) atomicAdd(&ctl->m_lvl[(d + 1) & 3], x);
    md = 0;
  };

  for (int d = 0;; ++d) {
    const unsigned long long qv = __ldcg(&ctl->qctr[d & 3]);
    const unsigned qn = (unsigned)(qv >> 32), qe = (unsigned)qv;
    if (qn == 0) break;
    const unsigned qn_prev = d > 0 ? (unsigned)(__ldcg(&ctl->qctr[(d + 3) & 3]) >> 32) : 0u;
    m_done += (long long)__ldcg(&ctl->m_lvl[d & 3]);
    const long long m_unseen = p.nnz_in - m_done;
    bool push;
    if (p.mode == TBFS_MODE_TOP_DOWN)
      push = true;
    else if (p.mode == TBFS_MODE_BOTTOM_UP)
      push = false;
    else
      push = (float)qe * p.alpha < (float)m_unseen + (float)kVCost * (float)n;
    if (tid == 0 && p.trace && d < p.trace_cap - 1) {
      long long *rec = p.trace + 4 * (long long)d;
      rec[0] = (long long)dev::global_ns();
      rec[1] = qn;
      rec[2] = qe;
      rec[3] = push ? 0 : 1;
    }
    if (tid == 0) {
      ctl->qctr[(d + 2) & 3] = 0ull;
      ctl->hctr[(d + 2) & 3] = 0ull;
      ctl->m_lvl[(d + 2) & 3] = 0ull;
      ctl->levels = d + 1;
      if (push)
        ctl->push_levels += 1;
      else
        ctl->pull_levels += 1;
    }
    const int b0 = d % 3, b1 = (d + 1) % 3, bm = (d + 2) % 3;
    const unsigned *Fd = p.F[b0];
    unsigned *F1 = p.F[b1];
    unsigned *Fm = p.F[bm];
    unsigned long long *qctr1 = &ctl->qctr[(d + 1) & 3];
    const unsigned nclear = (qn_prev + kClear - 1) / kClear;

    /* clear the rows of F_{d-1} (buffer of F_{d+2}) listed in Q_{d-1} */
    auto clear_item = [&](unsigned c) {
      for (unsigned j = g.lane; j < (unsigned)kClear; j += 32) {
        const unsigned idx = c * kClear + j;
        if (idx < qn_prev) {
          const int v = __ldcg(p.q[bm] + idx);
          unsigned z[W];
#pragma unroll
          for (int w = 0; w < W; ++w) z[w] = 0u;
          store_row<W>(Fm + (size_t)v * W, z);
        }
      }
    };

    if (push) {
      /* ---- phase 1: discovery over the out-edges of Q_d ---- */
      const unsigned nA = (qe + kPushRounds * 32 - 1) / (kPushRounds * 32);
      if (tid == 0) ctl->work[(ph + 2) & 3u] = 0u;
      first_claim = true;
      for (;;) {
        const unsigned it = claim(nA + nclear);
        if (it >= nA + nclear) break;
        if (it >= nA) {
          clear_item(it - nA);
          continue;
        }
        for (int r = 0; r < kPushRounds; ++r) {
          const unsigned t = it * (kPushRounds * 32) + r * 32 + g.lane;
          bool first = false;
          int v = 0;
          unsigned dgo = 0;
          if (t < qe) {
            const unsigned o = upper_owner(p.e[b0], qn, t);
            const int u = __ldcg(p.q[b0] + o);
            v = __ldg(p.jr + __ldg(p.rp + u) + (int)(t - __ldcg(p.e[b0] + o)));
            unsigned fr[W], sv[W];
            load_row<W>(Fd + (size_t)u * W, fr);
            load_row<W>(p.seen + (size_t)v * W, sv);
            bool any = false;
#pragma unroll
            for (int w = 0; w < W; ++w) {
              const unsigned m = fr[w] & ~sv[w];
              if (m) {
                atomicOr(&F1[(size_t)v * W + w], m);
                any = true;
              }
            }
            if (any) {
              const unsigned bit = 1u << (v & 31);
              first = (atomicOr(&p.touched[v >> 5], bit) & bit) == 0u;
              if (first) {
                dgo = (unsigned)(__ldg(p.rp + v + 1) - __ldg(p.rp + v));
                if (SIG) {
                  const int indeg = __ldg(p.cp + v + 1) - __ldg(p.cp + v);
                  if (indeg > p.seg_len) {
                    const unsigned long long old = atomicAdd(
                        &ctl->hctr[(d + 1) & 3],
                        (1ull << 32) | (unsigned long long)nsegs(indeg, p.seg_len));
                    p.hq[b1][old >> 32] = v;
                    p.he[b1][old >> 32] = (unsigned)old;
                  }
                }
              }
            }
          }
          warp_enqueue(first, v, dgo, p.q[b1], p.e[b1], qctr1);
        }
      }
      if (!grid_barrier(ctl, p.timeout_ns, d)) return;
      ++ph;

      /* ---- phase 2: path counts of the new vertices, finish them ---- */
      const unsigned qn1 = (unsigned)(__ldcg(qctr1) >> 32);
      const unsigned long long hv = SIG ? __ldcg(&ctl->hctr[(d + 1) & 3]) : 0ull;
      const unsigned hn1 = (unsigned)(hv >> 32), hsegs = (unsigned)hv;
      const unsigned qe1 = (unsigned)__ldcg(qctr1);
      const unsigned *e1 = p.e[b1];
      /* items of ~kItemCost list entries + vertex costs over the queue */
      const long long cost2 = (long long)qe1 + (long long)kVCost * qn1;
      const unsigned nA2 = (unsigned)((cost2 + kItemCost - 1) / kItemCost);
      const unsigned nB2 = (hsegs + PER - 1) / PER;
      auto qcost = [&](unsigned i) -> long long {
        return (long long)__ldcg(e1 + i) + (long long)kVCost * i;
      };
      if (tid == 0) ctl->work[(ph + 2) & 3u] = 0u;
      first_claim = true;
      for (;;) {
        const unsigned it = claim(nA2 + nB2);
        if (it >= nA2 + nB2) break;
        if (it < nA2) {
          const unsigned is = warp_lower_bound(qcost, qn1, (long long)it * kItemCost);
          const unsigned ie = warp_lower_bound(qcost, qn1, (long long)(it + 1) * kItemCost);
          for (unsigned base = is; base < ie; base += PER) {
            const unsigned idx = base + g.gid;
            bool full = false;
            int deg = 0;
            if (idx < ie) {
              const int v = __ldcg(p.q[b1] + idx);
              const int lo = __ldg(p.cp + v), hi = __ldg(p.cp + v + 1);
              deg = hi - lo;
              if (!SIG || deg <= p.seg_len) count_vertex<W, SIG>(p, d, v, lo, hi, Fd, F1, sm, g, full);
            }
            if (g.gl == 0 && full) md += (unsigned long long)deg;
          }
        } else if constexpr (SIG != 0) {
          const unsigned s = (it - nA2) * PER + g.gid;
          bool full = false;
          int deg = 0;
          if (s < hsegs) {
            const unsigned i = upper_owner(p.he[b1], hn1, s);
            const int h = __ldcg(p.hq[b1] + i);
            const unsigned si = s - __ldcg(p.he[b1] + i);
            const int cl = __ldg(p.cp + h), ch = __ldg(p.cp + h + 1);
            deg = ch - cl;
            const int lo = cl + (int)si * p.seg_len;
            const int hi = min(ch, lo + p.seg_len);
            count_segment<W, SIG>(p, d, h, lo, hi, nsegs(deg, p.seg_len), Fd, F1, sm, g, full);
          }
          if (g.gl == 0 && full) md += (unsigned long long)deg;
        }
      }
      flush_md(d);
      if (!grid_barrier(ctl, p.timeout_ns, d)) return;
      ++ph;
    } else {
      /* ---- pull: every vertex not reached by all roots ---- */
      const unsigned nA = ((unsigned)p.hub_segs + PER - 1) / PER;
      const long long cost = p.nnz_in + (long long)kVCost * n;
      const unsigned nB = (unsigned)((cost + kItemCost - 1) / kItemCost);
      auto vcost = [&](unsigned v) -> long long {
        return (long long)__ldg(p.cp + v) + (long long)kVCost * v;
      };
      if (tid == 0) ctl->work[(ph + 2) & 3u] = 0u;
      first_claim = true;
      for (;;) {
        const unsigned it = claim(nA + nB + nclear);
        if (it >= nA + nB + nclear) break;
        if (it >= nA + nB) {
          clear_item(it - nA - nB);
          continue;
        }
        unsigned bcnt = 0;
        /* hub item: one segment per group; vertex item: the vertices of
         * ~kItemCost list entries + vertex costs, PER at a time */
        unsigned vs = 0, ve = 1;
        if (it >= nA) {
          vs = warp_lower_bound(vcost, (unsigned)n, (long long)(it - nA) * kItemCost);
          ve = warp_lower_bound(vcost, (unsigned)n, (long long)(it - nA + 1) * kItemCost);
        }
        for (unsigned base = vs; base < ve; base += (it < nA ? 1u : (unsigned)PER)) {
          bool take = false, full = false;
          int v = 0, deg = 0;
          if (it < nA) {
            const unsigned s = it * PER + g.gid;
            if (s < (unsigned)p.hub_segs) {
              const unsigned i = upper_owner(p.hub_seg, (unsigned)p.nhub, s);
              v = __ldg(p.hubs + i);
              const unsigned si = s - (unsigned)__ldg(p.hub_seg + i);
              const int cl = __ldg(p.cp + v), ch = __ldg(p.cp + v + 1);
              deg = ch - cl;
              unsigned sn[W];
              load_row<W>(p.seen + (size_t)v * W, sn);
              bool done = true;
#pragma unroll
              for (int w = 0; w < W; ++w) done &= sn[w] == p.valid[w];
              if (!done) {
                const int lo = cl + (int)si * p.seg_len;
                const int hi = min(ch, lo + p.seg_len);
                pull_segment<W, SIG>(p, d, v, lo, hi, nsegs(deg, p.seg_len), sn, Fd, F1, sm, g,
                                     take, full);
              }
            }
          } else {
            const unsigned vv = base + g.gid;
            v = (int)vv;
            if (vv < ve) {
              const int lo = __ldg(p.cp + v), hi = __ldg(p.cp + v + 1);
              deg = hi - lo;
              if (deg <= p.seg_len) {
                unsigned sn[W];
                load_row<W>(p.seen + (size_t)v * W, sn);
                bool done = true;
#pragma unroll
                for (int w = 0; w < W; ++w) done &= sn[w] == p.valid[w];
                if (!done) pull_vertex<W, SIG>(p, d, v, lo, hi, sn, Fd, F1, sm, g, take, full);
              }
            }
          }
          const bool tk = g.gl == 0 && take;
          if (g.gl == 0 && full) md += (unsigned long long)deg;
          const unsigned bal = __ballot_sync(FULL, tk);
          if (tk) {
            const unsigned pos = bcnt + __popc(bal & ((1u << g.lane) - 1u));
            s_bv[wid][pos] = v;
            s_bd[wid][pos] = (unsigned)(__ldg(p.rp + v + 1) - __ldg(p.rp + v));
          }
          bcnt += __popc(bal);
          if (bcnt > 32u - PER) { /* the buffer could overflow next step: flush */
            __syncwarp();
            const bool ft = g.lane < (int)bcnt;
            warp_enqueue(ft, ft ? s_bv[wid][g.lane] : 0, ft ? s_bd[wid][g.lane] : 0u, p.q[b1],
                         p.e[b1], qctr1);
            __syncwarp();
            bcnt = 0;
          }
        }
        __syncwarp();
        const bool tk = g.lane < (int)bcnt;
        warp_enqueue(tk, tk ? s_bv[wid][g.lane] : 0, tk ? s_bd[wid][g.lane] : 0u, p.q[b1], p.e[b1],
                     qctr1);
        __syncwarp();
      }
      flush_md(d);
      if (!grid_barrier(ctl, p.timeout_ns, d)) return;
      ++ph;
    }
  }
  if (tid == 0 && p.trace) {
    const int slot = ctl->levels < p.trace_cap - 1 ? ctl->levels : p.trace_cap - 1;
    long long *rec = p.trace + 4 * (long long)slot;
    rec[0] = (long long)dev::global_ns();
    rec[1] = 0;
    rec[2] = 0;
    rec[3] = -1;
  }
}

/* ---- results: internal rows -> caller layout, per-root statistics ---------- */

template <int W, int SIG>
__global__ void __launch_bounds__(256) fm_output_kernel(const BatchOutParams o) {
  constexpr int RS = 32 * W;
  __shared__ int sS[32][33];
  __shared__ unsigned long long sG[SIG ? 32 : 1][33];
  __shared__ unsigned long long s_vis[8][32], s_edg[8][32];
  __shared__ int s_md[8][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int rb = blockIdx.y;
  const int r = rb * 32 + lane;
  const bool rv = r < o.k;
  unsigned long long vis = 0, edg = 0;
  int mdep = -1;
  const int ntiles = (o.n + 31) / 32;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int i0 = tile * 32;
    for (int j = wid; j < 32; j += 8) {
      const int i = i0 + j;
      int s = -1;
      unsigned long long cv = 0;
      if (i < o.n) {
        const int v = o.inv ? __ldg(o.inv + i) : i;
        const int rbit = bit_of_root(rv ? r : 0, W);
        const unsigned sw = __ldg(o.seen + (size_t)v * W + (rbit >> 5));
        if (rv && ((sw >> (rbit & 31)) & 1u)) {
          s = __ldg(o.S_int + (size_t)v * RS + r);
          if (SIG == 2) cv = __ldg(reinterpret_cast<const unsigned *>(o.sig_int) + (size_t)v * RS + r);
          else if (SIG) cv = __ldg(o.sig_int + (size_t)v * RS + r);
          ++vis;
          edg += (unsigned long long)(__ldg(o.rp + v + 1) - __ldg(o.rp + v));
          mdep = max(mdep, s);
        }
        if (o.layout == TBFS_LAYOUT_VERTEX_MAJOR && rv) {
          o.S_out[(size_t)i * o.ldo + r] = s;
          if (SIG && o.sig_out) o.sig_out[(size_t)i * o.ldo + r] = cv;
        }
      }
      if (o.layout == TBFS_LAYOUT_ROOT_MAJOR) {
        sS[lane][j] = s;
        if (SIG) sG[lane][j] = cv;
      }
    }
    if (o.layout == TBFS_LAYOUT_ROOT_MAJOR) {
      __syncthreads();
      for (int rr = wid; rr < 32; rr += 8) {
        const int root = rb * 32 + rr;
        if (root < o.k && i0 + lane < o.n) {
          o.S_out[(size_t)root * o.ldo + i0 + lane] = sS[rr][lane];
          if (SIG && o.sig_out) o.sig_out[(size_t)root * o.ldo + i0 + lane] = sG[rr][lane];
        }
      }
      __syncthreads();
    }
  }
  s_vis[wid][lane] = vis;
  s_edg[wid][lane] = edg;
  s_md[wid][lane] = mdep;
  __syncthreads();
  if (wid == 0 && rv) {
    unsigned long long a = 0, b = 0;
    int m = -1;
    for (int w = 0; w < 8; ++w) {
      a += s_vis[w][lane];
      b += s_edg[w][lane];
      m = max(m, s_md[w][lane]);
    }
    if (a) {
      atomicAdd(o.r_visited + r, a);
      atomicAdd(o.r_edges + r, b);
      atomicMax(o.r_maxd + r, m);
    }
  }
}

/* ---- hub list ------------------------------------------------------------------ */

__global__ void hub_flag_kernel(const int *cp, int n, int seg_len, int *flag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (cp[i + 1] - cp[i]) > seg_len ? 1 : 0;
  if (i == n) flag[n] = 0;
}

__global__ void hub_fill_kernel(const int *cp, int n, int seg_len, const int *pos, int *hubs,
                                int *nseg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pos[i + 1] != pos[i]) {
    hubs[pos[i]] = (int)i;
    nseg[pos[i]] = (int)nsegs(cp[i + 1] - cp[i], seg_len);
  }
}

template <int W>
const void *kernel_of(int sigma) {
  switch (sigma) {
    case 0: return reinterpret_cast<const void *>(fm_bfs_kernel<W, 0>);
    case 1: return reinterpret_cast<const void *>(fm_bfs_kernel<W, 1>);
    case 2: return reinterpret_cast<const void *>(fm_bfs_kernel<W, 2>);
    default: return nullptr;
  }
}

/* dynamic shared memory of the kernel: the path-count stage */
size_t stage_bytes(int sigma) {
  return sigma ? (size_t)kWarps * kStageU64 * sizeof(unsigned long long) : 0;
}

const void *batch_kernel(int W, int sigma) {
  switch (W) {
    case 1: return kernel_of<1>(sigma);
    case 2: return kernel_of<2>(sigma);
    case 4: return kernel_of<4>(sigma);
    case 8: return kernel_of<8>(sigma);
    default: return nullptr;
  }
}

}  // namespace

cudaError_t batch_hubs(const int *cp, int n, int seg_len, int **hubs, int **hub_seg, int *nhub,
                       int *hub_segs, cudaStream_t s) {
  *hubs = nullptr;
  *hub_seg = nullptr;
  *nhub = 0;
  *hub_segs = 0;
  int *pos = nullptr;
  cudaError_t e = tbfs::dev_alloc(&pos, ((size_t)n + 1) * sizeof(int));
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)(((long long)n + 1 + 255) / 256);
  hub_flag_kernel<<<blocks, 256, 0, s>>>(cp, n, seg_len, pos);
  if ((e = cudaGetLastError()) == cudaSuccess) e = exclusive_scan(pos, (long long)n + 1, pos, s);
  int cnt = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&cnt, pos + n, sizeof(int), cudaMemcpyDeviceToHost);
  int *h = nullptr, *ns = nullptr;
  if (e == cudaSuccess) e = tbfs::dev_alloc(&h, ((size_t)cnt + 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&ns, ((size_t)cnt + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(ns, 0, ((size_t)cnt + 1) * sizeof(int), s);
  if (e == cudaSuccess && cnt > 0) {
    hub_fill_kernel<<<(unsigned)(((long long)n + 255) / 256), 256, 0, s>>>(cp, n, seg_len, pos, h,
                                                                           ns);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = exclusive_scan(ns, (long long)cnt + 1, ns, s);
  int tot = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&tot, ns + cnt, sizeof(int), cudaMemcpyDeviceToHost);
  tbfs::dev_free(pos);
  if (e != cudaSuccess) {
    tbfs::dev_free(h);
    tbfs::dev_free(ns);
    return e;
  }
  *hubs = h;
  *hub_seg = ns;
  *nhub = cnt;
  *hub_segs = tot;
  return cudaSuccess;
}

cudaError_t batch_geometry(int device, int W, int sigma, LaunchGeom *out) {
  const void *k = batch_kernel(W, sigma);
  if (!k) return cudaErrorInvalidValue;
  int sms = 0, coop = 0, per = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (e != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  const size_t dyn = stage_bytes(sigma);
  if (dyn) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, kBlock, dyn);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  out->block = kBlock;
  out->grid = sms * per;
  return cudaSuccess;
}

cudaError_t batch_launch(const BatchParams &p, int W, int sigma, const LaunchGeom &g,
                         cudaStream_t s) {
  const void *k = batch_kernel(W, sigma);
  if (!k) return cudaErrorInvalidValue;
  void *args[] = {const_cast<BatchParams *>(&p)};
  return cudaLaunchCooperativeKernel(k, dim3(g.grid), dim3(g.block), args, stage_bytes(sigma), s);
}

template <int W>
void output_w(const BatchOutParams &o, int sigma, dim3 grid, cudaStream_t s) {
  if (sigma == 2) fm_output_kernel<W, 2><<<grid, 256, 0, s>>>(o);
  else if (sigma == 1) fm_output_kernel<W, 1><<<grid, 256, 0, s>>>(o);
  else fm_output_kernel<W, 0><<<grid, 256, 0, s>>>(o);
}

cudaError_t batch_output(const BatchOutParams &o, int sigma, cudaStream_t s) {
  const int ntiles = (o.n + 31) / 32;
  const dim3 grid((unsigned)min(ntiles, 4096), (unsigned)((o.k + 31) / 32));
  switch (o.W) {
    case 1: output_w<1>(o, sigma, grid, s); break;
    case 2: output_w<2>(o, sigma, grid, s); break;
    case 4: output_w<4>(o, sigma, grid, s); break;
    case 8: output_w<8>(o, sigma, grid, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tbfs
