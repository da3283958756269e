/*
 * tbfs_internal.h -- types shared by the engine's translation units.
 *
 * HBM layout of one resident graph (n vertices, nnz CSC entries):
 *   cp[n+1], ic[nnz]   int32 CSC: in-lists (column v = sources of edges ->v)
 *   rp[n+1], jr[nnz]   int32 out-lists; aliases cp/ic when the graph is
 *                      symmetric, else the transpose built on the device
 * Per-traversal workspace (reused across calls on the same graph), three
 * rotating buffers so that the queues of levels d-1, d and d+1 coexist:
 *   q[3][n]            int32 frontier vertices
 *   e[3][n]            int32 out-edge offset of each queue entry (exclusive
 *                      prefix of out-degrees, in queue order)
 *   a[3][n]            int32 start of each queue entry's out-list (rp[v])
 *   fb[4][n/32]        frontier bitmaps (bit v of fb[d % 4]: v in F_d); four so
 *                      that F_{d-1} and F_d are read while F_{d+1} is written
 *                      and F_{d+2}'s is cleared in the same phase
 *   ctl                control block: per-level counters, barrier words
 * Outputs: S[n] int32 (-1 unreached), sigma[n] uint64 bit patterns of the
 * int64 path counts.
 */
#ifndef TBFS_INTERNAL_H
#define TBFS_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "tbfs.h"

namespace tbfs {

/* Device memory of the library (devmem.cu): a stream-ordered pool per GPU.
 * dev_alloc's block is usable from every stream on return; dev_free waits
 * for the device like cudaFree, then hands the block back to the pool. */
cudaError_t dev_alloc(void **p, size_t bytes);
cudaError_t dev_free(void *p);
cudaError_t dev_trim(size_t keep);
template <class T>
inline cudaError_t dev_alloc(T **p, size_t bytes) {
  return dev_alloc(reinterpret_cast<void **>(p), bytes);
}

/* Arrival counter of the hand-written grid barrier (device_common.cuh), on
 * its own 128-byte line. */
struct __align__(128) GridBarrier {
  unsigned arrive;
  unsigned pad0[31];
};

/* Device control block of one traversal; zeroed before every launch. */
struct __align__(128) BfsCtl {
  /* slot d % 3 accumulates the queue of level d+1 ... see bfs_engine.cu */
  unsigned long long qctr[3];
  int status;          /* TBFS_OK or TBFS_ERR_TIMEOUT                     */
  int sigma_overflow;  /* some path count passed INT64_MAX               */
  int levels, td_levels, bu_levels;
  int timeout_level;   /* level + 2 of the barrier that gave up, else 0  */
  long long visited, edges;
  unsigned int work[4]; /* dynamic work counter of phase d in work[d % 4] */
  unsigned int pad0[10];
  GridBarrier bar;
};

struct BfsParams {
  const int *cp, *ic; /* in-lists  */
  const int *rp, *jr; /* out-lists */
  int *S;
  unsigned long long *sigma; /* null: S only */
  int *q[3], *e[3], *a[3];   /* queue buffers; level d uses buffer d % 3 */
  unsigned *fb[4];           /* frontier bitmaps; F_d in fb[d % 4]         */
  BfsCtl *ctl;
  long long out_edges_total;
  long long timeout_ns;
  int n, root, mode, symmetric;
  float alpha, beta;
  float pull_ratio; /* see tbfs_options.pull_ratio */
  int inject_barrier_skip; /* test hook, 0 = off */
  int trace_cap;           /* records in trace */
  long long *trace;        /* device buffer of trace_cap x 4 int64, or null */
  /* graph stored in its own numbering: inv[caller id] = internal id,
   * perm[internal id] = caller id; S and sigma above are then internal work
   * arrays, scattered into S_out / sigma_out (caller order) at the end.
   * Null: identity. */
  const int *inv;
  const int *perm;
  int *S_out;
  unsigned long long *sigma_out;
  /* engine shape: most list entries per lane and round (0: the compiled
   * maximum), CTAs per SM of the launch (0: as many as fit) */
  int max_ept;
  int ctas_per_sm;
  /* bits of the largest in-degree (0: unknown); bounds the path counts'
   * growth per level (bfs_engine.cu) */
  int deg_bits;
  /* nonzero: no out-list has more than kShortList entries, so small
   * top-down levels may give every queue entry to one lane (bfs_engine.cu) */
  int short_lists;
};

/* longest out-list for which a lane walks a whole list alone */
constexpr int kShortList = 16;

/* Control block of a COOC traversal (cooc_engine.cu); zeroed before every
 * launch. */
struct __align__(128) CoocCtl {
  unsigned long long cnt[3]; /* vertices of level d in cnt[d % 3] */
  int status, timeout_level;
  int levels;
  int sigma_overflow;
  int unfinished;            /* gave up after max_levels levels */
  int pad0[21];
  GridBarrier bar;
};

struct CoocParams {
  const int *I, *J;          /* entry k: edge I[k] -> J[k] */
  long long nnz;
  int n, root;
  int vec;                   /* I and J 16-byte aligned: four pairs per load */
  int max_levels;
  int *S;
  unsigned long long *sigma; /* null: depths only */
  unsigned *fb[3];           /* frontier bitmaps, (n + 31) / 32 words each */
  CoocCtl *ctl;
  long long timeout_ns;
};

/* Launch geometry of the persistent kernel on the current device. */
struct LaunchGeom {
  int grid = 0;
  int block = 0;
  int sms = 0, per_sm = 0; /* grid = sms * per_sm */
};

cudaError_t bfs_launch(const BfsParams &p, const LaunchGeom &g, cudaStream_t s);
cudaError_t bfs_geometry(int device, LaunchGeom *out);
cudaError_t cooc_geometry(int device, LaunchGeom *out);
cudaError_t cooc_launch(const CoocParams &p, const LaunchGeom &g, cudaStream_t s);
/* *d_flag = 1 when some I[k] or J[k] is outside [0, n) */
cudaError_t cooc_check(const int *I, const int *J, long long nnz, int n, int *d_flag,
                       cudaStream_t s);
/* *out = the longest list of the n lists delimited by ptr[0..n] (ptr on the
 * device), synchronously on the current device */
cudaError_t longest_list(const int *ptr, int n, int *out);

/* ---- frontier-matrix batch (batch_engine.cu) ----
 * Up to 256 roots on one graph advance together: bit r of a vertex's row
 * stands for root r.  Rows are W 32-bit words (W in {1, 2, 4, 8}, 32 W >=
 * roots of the launch); per-root values are rows of 32 W entries. */
constexpr int kBatchMaxRoots = 256;

struct __align__(128) BatchCtl {
  unsigned long long qctr[4]; /* Q_d: (count << 32) | out-edge sum, slot d % 4   */
  unsigned long long hctr[4]; /* hub part of Q_d: (count << 32) | segments       */
  unsigned long long m_lvl[4]; /* in-list entries of vertices all roots reached
                                  during level d - 1, slot d % 4              */
  unsigned work[4];           /* dynamic work counter of phase ph in work[ph % 4] */
  int status, timeout_level;
  int levels, push_levels, pull_levels;
  int wide; /* a launch with 32-bit counts met a count that needs more bits */
  unsigned ovf[8]; /* bit r: a path count of root r reached 2^63 */
  unsigned pad1[2];
  GridBarrier bar;
};

struct BatchParams {
  const int *cp, *ic; /* in-lists (pull)  */
  const int *rp, *jr; /* out-lists (push) */
  int n;
  long long nnz_in;   /* in-list entries (direction rule) */
  int k;              /* roots of this launch (<= 256)      */
  const int *roots;   /* root r: caller vertex id (k)       */
  const int *inv;     /* caller id -> internal id, or null  */
  unsigned *seen;     /* [n][W]: roots that reached v       */
  unsigned *F[3];     /* [n][W]: F_d in F[d % 3]            */
  int *q[3];          /* frontier queue of level d in q[d % 3] ...      */
  unsigned *e[3];     /* ... with the exclusive prefix of out-degrees   */
  int *hq[3];         /* hub entries of the queue (vertex) ...          */
  unsigned *he[3];    /* ... with the exclusive prefix of segment counts */
  unsigned *touched;  /* [ceil(n/32)] queue membership during push levels */
  unsigned *seg_arrive; /* [n] cumulative segment arrivals (hubs)         */
  int *S_int;         /* [n][32W] depth of v from root r (valid where seen) */
  unsigned long long *sig_int; /* [n][32W] path counts (uint64; uint32 in the
                                  kernels with 32-bit counts), or null        */
  const int *hubs;    /* vertices with more than seg_len in-list entries   */
  const int *hub_seg; /* exclusive prefix of their segment counts (nhub+1) */
  int nhub;
  int hub_segs;
  int seg_len;
  BatchCtl *ctl;
  long long timeout_ns;
  float alpha;
  int mode;           /* TBFS_MODE_*: AUTO, TOP_DOWN (push), BOTTOM_UP (pull) */
  unsigned valid[8];  /* root bits in use, per word */
  long long *trace;   /* trace_cap x 4 records {ns, |Q_d|, out-edges, 0 push / 1 pull}, or null */
  int trace_cap;
};

struct BatchOutParams {
  int n, k, W, layout;
  long long ldo;      /* output row stride: n (root-major) or the caller's k */
  const int *inv;     /* caller id -> internal id, or null */
  const int *rp;      /* out-degrees for the per-root edge counts */
  const unsigned *seen;
  const int *S_int;
  const unsigned long long *sig_int;
  int *S_out;                  /* root r, caller id i at r * ldo + i (root-major)
                                  or i * ldo + r (vertex-major) */
  unsigned long long *sig_out; /* same layout, or null        */
  unsigned long long *r_visited, *r_edges; /* per-root stats (k) */
  int *r_maxd;
};

/* Graph-wide hub list for segment length seg_len: hubs (nhub) and hub_seg
 * (nhub + 1, exclusive prefix of ceil(indeg / seg_len)), allocated here. */
cudaError_t batch_hubs(const int *cp, int n, int seg_len, int **hubs, int **hub_seg, int *nhub,
                       int *hub_segs, cudaStream_t s);
/* sigma: 0 depths only, 1 64-bit path counts, 2 32-bit path counts (the
 * launch sets ctl->wide when a count needs more bits; it is then redone
 * with 1) */
cudaError_t batch_geometry(int device, int W, int sigma, LaunchGeom *out);
cudaError_t batch_launch(const BatchParams &p, int W, int sigma, const LaunchGeom &g,
                         cudaStream_t s);
cudaError_t batch_output(const BatchOutParams &o, int sigma, cudaStream_t s);

struct BatchWS; /* per-graph batch workspace (batch_api.cu) */
void batch_ws_free(BatchWS *ws);

/* ---- multi-instance engine (multi_engine.cu) ----
 * One descriptor per traversal (graph, root); the kernel advances every
 * unfinished descriptor by one level per phase. */
constexpr int kMultiMaxSlots = 1024;

struct InstDesc {
  const int *cp, *ic;         /* in-lists  */
  const int *rp, *jr;         /* out-lists (the pushes walk these) */
  const int *inv;             /* caller id -> internal id, or null */
  long long nnz;
  int n;
  int root;                   /* caller numbering */
  int *S;                     /* n depths (internal numbering), -1 initially  */
  unsigned long long *sig;    /* n path counts, 0 initially; null: depths only */
  int *q[3];                  /* frontier queue of level d in q[d % 3] ...     */
  unsigned *e[3];             /* ... with the exclusive prefix of out-degrees */
  unsigned long long ctr[3];  /* queue of level d: (count << 32) | out-edges   */
  int d;                      /* next level to run                             */
  int done;                   /* 1: finished (or an empty slot)                */
  int levels;
  int ovf;                    /* a path count reached 2^63                     */
  int deg_bits;               /* bits of the largest in-degree (0: unknown):
                                 counts of level d have at most 1 + d deg_bits */
  long long visited, edges;
};

struct __align__(128) MultiCtl {
  unsigned work[4];
  int status, timeout_level;
  int phases;                 /* levels run by the launch */
  int stop[2];                /* end the launch after level ph: stop[ph % 2], written
                                 during the level, read after its barrier; two slots
                                 so that a CTA already in level ph+1 cannot write
                                 the word a slower CTA is still to read for ph */
  int pad0[23];
  GridBarrier bar;
};

struct MultiParams {
  InstDesc *inst;
  int nslots;                 /* descriptors (<= kMultiMaxSlots) */
  int max_phases;             /* stop after this many levels     */
  MultiCtl *ctl;
  long long timeout_ns;
  const volatile int *wake;   /* host-mapped flag: requests wait (null: none) */
  int stop_on_done;           /* end the launch after a level that finished an instance */
};

cudaError_t multi_geometry(int device, LaunchGeom *out);
cudaError_t multi_launch(const MultiParams &p, const LaunchGeom &g, cudaStream_t s);
/* initialise the descriptors slots[0..k) (S = -1 and sig = 0 already set) */
cudaError_t multi_init(InstDesc *inst, const int *slots, int k, cudaStream_t s);
/* out[j] = S[inv[j]] (or S[j]) for j < n; sig likewise when sig_out is set */
cudaError_t multi_gather(const int *S, const unsigned long long *sig, const int *inv, int n,
                         int *S_out, unsigned long long *sig_out, cudaStream_t s);

/* graph ingest helpers (graph_ingest.cu) */
cudaError_t validate_csc(const int *cp, const int *ic, int n, long long nnz,
                         int *d_flag, cudaStream_t s);
/* (key, val) pairs -> ptr[n+1] / idx[nnz] lists, each list in the input
 * order of its entries; a key outside [0, n) sets bit 2 of *d_flag (and the
 * lists are then not built), a value outside it too */
cudaError_t counting_sort_lists(const int *keys, const int *vals, long long nnz,
                                int n, int *ptr_out, int *idx_out, int *d_flag,
                                cudaStream_t s);
/* stable LSD radix sort of len (key, val) pairs by the low `bits` bits of
 * the key; ktmp / vtmp are len-element scratch; synchronises s */
cudaError_t stable_sort_pairs(unsigned *keys, unsigned *vals, long long len, int bits,
                              unsigned *ktmp, unsigned *vtmp, cudaStream_t s);
/* bits needed for keys up to max_key */
int key_bits(unsigned max_key);

/* device edge list -> CSC (cp[n+1], ic[nnz], allocated here) with the host
 * builder's construction flags (TBFS_BUILD_*); *bad = 1 when an endpoint is
 * outside [0, n).  cudaErrorInvalidValue: more than INT32_MAX pairs.
 * (mm_ingest.cu) */
cudaError_t csc_from_edges_device(const int *src, const int *dst, long long m, int n,
                                  unsigned flags, int **cp_out, int **ic_out, long long *nnz_out,
                                  int *bad_out, cudaStream_t s);
/* the data lines of a Matrix Market coordinate file (len bytes on the
 * device, starting at a line) -> src/dst of the first nz entries;
 * *lines = data lines found, *bad = first entry that is not two indices in
 * range (or -1) */
cudaError_t mm_parse_device(const char *text, long long len, long long nz, long long M,
                            long long N, int *src, int *dst, long long *lines_out,
                            long long *bad_out, cudaStream_t s);
/* exclusive prefix sum of len ints (in place allowed); synchronises s */
cudaError_t exclusive_scan(const int *in, long long len, int *out, cudaStream_t s);
/* the same queued on s without synchronising, with the caller's scratch of
 * scan_partials(len) ints */
long long scan_partials(long long len);
cudaError_t exclusive_scan_ws(const int *in, long long len, int *out, int *partial,
                              cudaStream_t s);
cudaError_t expand_columns(const int *cp, int n, int *col_of_entry, cudaStream_t s);
/* Whether the CSC (validated) equals its transpose as a multiset of entries:
 * the sums over all entries u -> v of h(u, v) - h(v, u) vanish for two
 * keyed 64-bit hashes (keys chosen by the caller at random).  A graph that
 * is its own transpose always passes; any other passes only when both
 * independent sums cancel by chance (about 2^-128 for random keys). */
cudaError_t symmetric_check(const int *cp, const int *ic, int n, long long nnz,
                            unsigned long long key1, unsigned long long key2, bool *symmetric,
                            cudaStream_t s);
/* Degree-based grouping of the vertices (see graph_ingest.cu).  On return
 * *identity tells whether the order is unchanged (then perm/inv/cp2/ic2 are
 * untouched); otherwise perm[new] = old, inv[old] = new and (cp2, ic2) is the
 * CSC with columns and row ids renamed. */
cudaError_t degree_group_relabel(const int *cp, const int *ic, int n, long long nnz,
                                 int *perm, int *inv, int *cp2, int *ic2, bool *identity,
                                 cudaStream_t s);

}  // namespace tbfs

struct tbfs_graph {
  int device = 0;
  int32_t n = 0;
  int64_t nnz = 0;
  uint32_t flags = 0;
  int *cp = nullptr, *ic = nullptr;
  int *rp = nullptr, *jr = nullptr;
  bool separate_out = false;
  long long out_edges_total = 0;
  /* workspace */
  int *queues = nullptr; /* one allocation: q[3], e[3], a[3], n ints each */
  char *hot = nullptr;   /* one allocation: sigma_work, S_work, bitmaps */
  int deg_bits = 0;      /* bits of the largest in-degree */
  bool short_lists = false; /* no out-list longer than kShortList */
  /* the caller's TBFS_GRAPH_SYMMETRIC (flags may also carry it when the
   * lists were found to equal their transpose on upload) */
  bool declared_symmetric = false;
  unsigned *bitmaps = nullptr; /* four frontier bitmaps, (n+31)/32 words each */
  /* degree-grouped numbering: inv[caller id] = internal id (null: identity);
   * the traversal works on internal S/sigma and un-permutes at the end */
  int *inv = nullptr;
  int *perm = nullptr; /* perm[internal id] = caller id */
  int *S_work = nullptr;
  unsigned long long *sigma_work = nullptr;
  tbfs::BfsCtl *ctl = nullptr;
  tbfs::BfsCtl *ctl_host = nullptr; /* pinned mirror */
  int *S_dev = nullptr;
  unsigned long long *sigma_dev = nullptr;
  /* second result buffer and a copy stream: tbfs_bfs_many with host outputs
   * copies root i's results back while root i+1 is traversed */
  int *S_dev2 = nullptr;
  unsigned long long *sigma_dev2 = nullptr;
  cudaStream_t copy_stream = nullptr;
  long long *trace_dev = nullptr; /* per-level trace records */
  int trace_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t last_stream = nullptr;
  tbfs::LaunchGeom geom;
  tbfs::BatchWS *batch = nullptr; /* frontier-matrix workspace, on first use */
  /* tbfs_bfs_many: one control block per root (cleared together, read back
   * together) and two events per root, kept for the next call */
  tbfs::BfsCtl *many_ctl = nullptr;
  tbfs::BfsCtl *many_ctl_host = nullptr; /* pinned */
  int many_cap = 0;
  std::vector<cudaEvent_t> many_ev;   /* 2 per root, timing          */
  std::vector<cudaEvent_t> many_sync; /* 2 per root, ready / copied  */
  int depth_hint = 0; /* levels of the last traversal of this graph (0: none yet) */
  bool pending = false; /* a traversal was enqueued and not yet collected */
  tbfs_stats last = {};
};

namespace tbfs {
/* one traversal with results in the internal numbering (api.cu) */
tbfs_status forward_internal(tbfs_graph *g, int32_t root, const tbfs_options &o, int *S,
                             unsigned long long *sigma, cudaStream_t s, BfsCtl *ctl_host);
}  // namespace tbfs

extern "C" void tbfs_set_error(const char *fmt, ...);

#endif
