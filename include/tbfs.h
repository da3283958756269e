/*
 * tbfs.h -- native C ABI of the GB300 (sm_103a) linear-algebra BFS engine.
 *
 * The engine computes, for an unweighted graph held as a CSC adjacency
 * (column v lists the in-neighbours u of v, i.e. edge u->v) and a root r:
 *   S[v]     depth of v (root = 0, unreached = -1),
 *   sigma[v] number of shortest paths r->v, counted with the multiplicity of
 *            the CSC entries (int64; overflow past INT64_MAX is reported in
 *            tbfs_stats.sigma_overflow instead of being rounded).
 * These are the depth vector S and the path-count vector sigma of the
 * reference's semiring BFS (TurboBFS_CSC_TD/bfstdcsc_seq.c:48-80 and
 * TurboBFS_CSC_TD/spmvcsc_seq.c:22-41); both are unique functions of
 * (graph, root), so every traversal direction returns identical values.
 *
 * The reference's own entry points (bfs_gpu_td_csc_sc and friends) are
 * declared in tbfs_compat.h; the host graph tools in tbfs_graphgen.h.
 *
 * Threading: one tbfs_graph may be used by one host thread at a time.
 * Every call returns a tbfs_status; nothing in the library calls exit().
 */
#ifndef TBFS_H
#define TBFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TBFS_VERSION 100

typedef enum tbfs_status {
  TBFS_OK = 0,
  TBFS_ERR_INVALID_ARG = 1,   /* bad size, root out of range, null pointer  */
  TBFS_ERR_CUDA = 2,          /* a CUDA runtime call failed                 */
  TBFS_ERR_OUT_OF_MEMORY = 3, /* device or host allocation failed           */
  TBFS_ERR_TIMEOUT = 4,       /* a grid barrier wait ran past its budget    */
  TBFS_ERR_NO_DEVICE = 5,     /* no CUDA device visible                     */
  TBFS_ERR_IO = 6,            /* file could not be read / parsed            */
  TBFS_ERR_UNSUPPORTED = 7    /* valid request the library cannot serve     */
} tbfs_status;

typedef enum tbfs_mode {
  TBFS_MODE_AUTO = 0,      /* direction-optimizing, switched on the device */
  TBFS_MODE_TOP_DOWN = 1,  /* push from the frontier queue every level     */
  TBFS_MODE_BOTTOM_UP = 2  /* pull into unvisited vertices every level     */
} tbfs_mode;

/* tbfs_graph_create_* flags */
#define TBFS_GRAPH_SYMMETRIC 0x1u   /* caller guarantees in-lists == out-lists */
#define TBFS_GRAPH_DEVICE_PTRS 0x2u /* input arrays are device pointers       */
#define TBFS_GRAPH_KEEP_ORDER 0x4u  /* do not regroup vertices by degree; by
                                       default hub vertices are renumbered to
                                       the front inside the library (results
                                       are always in the caller's numbering) */

typedef struct tbfs_graph tbfs_graph;

typedef struct tbfs_options {
  int32_t mode;              /* tbfs_mode                                    */
  int32_t want_sigma;        /* 0: S only; 1: S and sigma                    */
  int32_t outputs_on_device; /* 1: S/sigma are device pointers               */
  int32_t inject_barrier_skip; /* testing: k > 0 makes one CTA leave before
                                  the barrier that ends level k-1, so the
                                  others' bounded waits expire and the call
                                  returns TBFS_ERR_TIMEOUT; 0 = off          */
  float alpha;               /* TD->BU when frontier edges > unexplored/alpha */
  float beta;                /* BU->TD when frontier size < n/beta           */
  void *stream;              /* cudaStream_t; NULL = legacy default stream   */
  int64_t timeout_ns;        /* grid-barrier wait budget; <=0 = 2 s          */
  /* Per-level trace (host memory, may be NULL): record d holds
   * {start ns (device globaltimer), frontier vertices, frontier out-edges,
   *  direction 0 = top-down / 1 = bottom-up}; one extra record {end ns, 0,
   *  0, -1} closes the run.  Capacity counts records (4 int64 each). */
  int64_t *level_trace;
  int32_t level_trace_cap;
  /* Path counts of a level found bottom-up are finished one level later,
   * either by pulling over that level's lists or by pushing from the
   * previous level's lists; pull is used unless it reads more than
   * pull_ratio times as many list entries as push.  <= 0: default 1. */
  float pull_ratio;
  /* Engine shape of the single-source traversal (tbfs_autotune sets both):
   * the most list entries a lane handles per round of a push or pull (1..6;
   * 0 = 6), and CTAs per SM of the persistent launch (0 = as many as fit,
   * or 2 on graphs whose out-lists all have at most 16 entries). */
  int32_t max_ept;
  int32_t ctas_per_sm;
} tbfs_options;

typedef struct tbfs_stats {
  int32_t levels;          /* non-empty BFS levels (max depth + 1)           */
  int32_t td_levels;       /* levels expanded top-down                       */
  int32_t bu_levels;       /* levels expanded bottom-up                      */
  int32_t sigma_overflow;  /* 1 if some path count exceeded INT64_MAX         */
  int64_t visited;         /* vertices reached, root included                */
  int64_t edges;           /* sum of out-degrees of reached vertices         */
  double device_ms;        /* CUDA-event time of the traversal on the stream */
} tbfs_stats;

/* Defaults: AUTO, want_sigma = 1, host outputs, alpha = 15, beta = 2,
 * pull_ratio = 1 (near the best of RMAT scale 18-22 and Erdos-Renyi scale 22
 * with path counts; Beamer's beta = 18 kept bottom-up levels after the
 * frontier had begun to shrink, 14-43 % slower on those graphs). */
void tbfs_options_init(tbfs_options *opt);

/* Upload a CSC adjacency (col_ptr[n+1], row_idx[nnz], int32, 0-based).
 * The graph stays resident until tbfs_graph_destroy.  Without
 * TBFS_GRAPH_SYMMETRIC the device first tests whether the lists equal their
 * transpose (the sums over the entries u -> v of h(u, v) - h(v, u) vanish
 * for two 64-bit hashes with fresh random keys; a graph that is not its own
 * transpose passes with probability about 2^-128): if so the in-lists serve
 * as out-lists and tbfs_graph_info reports TBFS_GRAPH_SYMMETRIC, otherwise
 * the transpose (out-lists) is built on the device. */
tbfs_status tbfs_graph_create_csc(const int32_t *col_ptr, const int32_t *row_idx,
                                  int32_t n, int64_t nnz, uint32_t flags,
                                  tbfs_graph **out);

/* Upload a COOC adjacency: entry k is the edge row[k] -> col[k] (the
 * reference's ICOOC/JCOOC, TurboBFS_COOC_TD/bfstdcooc.h:29-32).  Column order
 * is not required; the column pointer is rebuilt on the device. */
tbfs_status tbfs_graph_create_cooc(const int32_t *row, const int32_t *col,
                                   int32_t n, int64_t nnz, uint32_t flags,
                                   tbfs_graph **out);

/* Build a graph on the device from an edge list: edge k is src[k] ->
 * dst[k] (0-based), landing in column dst[k].  build_flags are those of the
 * host builder tbfs_csc_from_edges (tbfs_graphgen.h: TBFS_BUILD_SYMMETRIZE,
 * _DROP_LOOPS, _DEDUP, _SORT) and give the same col_ptr / row_idx: without
 * SORT or DEDUP a column keeps the input order of its entries.  Replaces
 * the reference's host builders CP_RP_ug / SSCCSC_uw / SSCCOOC_uw
 * (TurboBFS_CSC_TD/sparseformatransf.c:60-104,
 * TurboBFS_COOC_TD/sparseformatransf.c:62-95) for large graphs.
 * graph_flags as for tbfs_graph_create_csc (TBFS_GRAPH_SYMMETRIC is implied
 * by SYMMETRIZE; TBFS_GRAPH_DEVICE_PTRS: src/dst are device pointers). */
tbfs_status tbfs_graph_create_edges(const int32_t *src, const int32_t *dst, int32_t n,
                                    int64_t m, uint32_t build_flags, uint32_t graph_flags,
                                    tbfs_graph **out);

/* Parse Matrix Market coordinate text (a .mtx file's bytes in host memory)
 * on the device and build the graph from it: entry line k "i j [...]" is
 * the edge i-1 -> j-1; undirected adds each entry's mirror (a diagonal entry
 * twice), as the reference's readMMfile_uw + CP_RP_ug
 * (TurboBFS_CSC_TD/readMMfilef.c:56-70) and the host reader tbfs_mm_read do.
 * Errors (TBFS_ERR_IO): no banner, not coordinate, no size line, fewer
 * entry lines than the size line's nz, an index out of range. */
tbfs_status tbfs_graph_create_mm(const char *text, int64_t bytes, int32_t undirected,
                                 uint32_t build_flags, uint32_t graph_flags, tbfs_graph **out);

/* tbfs_graph_create_mm on the contents of a file (read into pinned memory). */
tbfs_status tbfs_graph_load_mm(const char *path, int32_t undirected, uint32_t build_flags,
                               uint32_t graph_flags, tbfs_graph **out);

/* Copy the resident in-lists (col_ptr[n+1], row_idx[nnz]) to the host.
 * TBFS_ERR_UNSUPPORTED for a graph stored regrouped by degree (create it
 * with TBFS_GRAPH_KEEP_ORDER to read it back). */
tbfs_status tbfs_graph_get_csc(const tbfs_graph *g, int32_t *col_ptr, int32_t *row_idx);

/* The same lists as COOC pairs row[k] -> col[k] (nnz each, in column order:
 * the reference's ICOOC / JCOOC, TurboBFS_COOC_TD/bfstdcooc.h:29-32), the
 * column of every entry expanded on the device. */
tbfs_status tbfs_graph_get_cooc(const tbfs_graph *g, int32_t *row, int32_t *col);

void tbfs_graph_destroy(tbfs_graph *g);

tbfs_status tbfs_graph_info(const tbfs_graph *g, int32_t *n, int64_t *nnz,
                            uint32_t *flags);

/* One BFS from root.  S must hold n int32; sigma n int64 (may be NULL when
 * want_sigma = 0).  stats may be NULL.  Synchronous unless outputs are on
 * the device, in which case it returns after enqueueing on opt->stream;
 * stats->device_ms is then filled by tbfs_graph_last_stats after a sync. */
tbfs_status tbfs_bfs(tbfs_graph *g, int32_t root, const tbfs_options *opt,
                     int32_t *S, int64_t *sigma, tbfs_stats *stats);

/* Check a BFS result against the graph (a validation in the manner of the
 * Graph500 benchmark's, run on the device).  The reference checks its GPU
 * output by comparing it with its own sequential BFS (S_check / bfs_check,
 * TurboBFS_CSC_TD/utils_bfs.c:93-145); S and sigma are the unique depth and
 * path-count vectors of (g, root) exactly when no violation below is found,
 * so this check needs no second traversal.  S (n int32, caller numbering)
 * and sigma (n int64, may be NULL to check depths only) are device pointers
 * when on_device, else host arrays (copied in).  Counts land in *out;
 * TBFS_OK means the check ran, not that it passed.  Synchronous on stream
 * (NULL = legacy default stream). */
typedef struct tbfs_validation {
  int64_t bad_root;       /* S[root] != 0, sigma[root] != 1, or another vertex at depth 0 */
  int64_t bad_depth;      /* S[v] < -1                                            */
  int64_t skips_level;    /* entries u->v with u reached and v unreached or
                             S[v] > S[u] + 1                                      */
  int64_t no_parent;      /* reached v != root without an in-neighbour at S[v]-1  */
  int64_t sigma_mismatch; /* sigma[v] != sum of its parents' sigma (mod 2^64), or
                             != 0 for an unreached v                              */
  int64_t first_bad;      /* smallest vertex with a violation, -1 if none         */
  int64_t visited;        /* vertices with S >= 0                                 */
  int64_t edges;          /* in-list entries of those vertices                    */
} tbfs_validation;
tbfs_status tbfs_bfs_validate(tbfs_graph *g, int32_t root, const int32_t *S,
                              const int64_t *sigma, int32_t on_device, void *stream,
                              tbfs_validation *out);

/* Statistics of the most recent traversal on g (synchronizes its stream). */
tbfs_status tbfs_graph_last_stats(tbfs_graph *g, tbfs_stats *stats);

/* k BFS runs, one per root, back to back on one stream.  Row i of the
 * outputs (stride n) receives root i's result; stats[i] likewise. */
tbfs_status tbfs_bfs_many(tbfs_graph *g, const int32_t *roots, int32_t k,
                          const tbfs_options *opt, int32_t *S, int64_t *sigma,
                          tbfs_stats *stats);

/* Many roots on one graph in one frontier-matrix traversal: up to 256 roots
 * advance together in one persistent launch (more are taken 256 at a time),
 * every list read shared by all of them.  No counterpart in the reference,
 * which runs one root per call; results are identical to k calls of
 * tbfs_bfs (S: -1 unreached; sigma: exact int64 path counts, per-root
 * overflow flag in stats[r].sigma_overflow).  Layout of S (k x n int32) and
 * sigma (k x n int64, may be NULL for depths only):
 *   TBFS_LAYOUT_ROOT_MAJOR    S[r * n + v]  (as tbfs_bfs_many)
 *   TBFS_LAYOUT_VERTEX_MAJOR  S[v * k + r]
 * Host or device outputs as opt->outputs_on_device; opt->mode AUTO picks
 * push or pull per level, TOP_DOWN / BOTTOM_UP force one; opt->alpha is the
 * push/pull threshold.  stats (may be NULL) receives k records; td_levels /
 * bu_levels count the batch's push / pull levels and device_ms is the time
 * of the launch that computed the root. */
#define TBFS_LAYOUT_ROOT_MAJOR 0
#define TBFS_LAYOUT_VERTEX_MAJOR 1
#define TBFS_BATCH_MAX_ROOTS 256
tbfs_status tbfs_bfs_batch(tbfs_graph *g, const int32_t *roots, int32_t k,
                           const tbfs_options *opt, int32_t layout, int32_t *S,
                           int64_t *sigma, tbfs_stats *stats);

/* Degree profile of a resident graph, computed on the device: hist40[b] =
 * vertices whose in-degree d has floor(log2(d+1)) == b (b < 40), the maximum
 * and the mean in-degree (the statistics of the reference's degree.c:22-141;
 * the same definition as tbfs_degree_profile of tbfs_graphgen.h on a host
 * CSC).  max_degree and mean_degree may be NULL. */
tbfs_status tbfs_graph_degree_profile(tbfs_graph *g, int64_t *hist40, int64_t *max_degree,
                                      double *mean_degree);

/* Degree statistics of a resident graph, the numbers the reference's
 * drivers print (TurboBFS_CSC_TD/degree.c:22-141, called from
 * TurboBFS_CSC_TD/bfstdcsc_main.c:177-260), computed on the device.  kind:
 *   TBFS_DEGREE_IN          in-degree (column lengths)
 *   TBFS_DEGREE_OUT         out-degree (row counts)
 *   TBFS_DEGREE_UNDIRECTED  degree_ug's out + in of the graph's entries: the
 *                           column length of a graph created with
 *                           TBFS_GRAPH_SYMMETRIC (or built symmetrised),
 *                           in + out otherwise
 * max_degree / argmax: degree_max (the first vertex, caller numbering, of
 * maximum degree; -1 when every degree is 0).  mean / sd: degree_sta (sum in
 * int64, sample standard deviation with divisor n - 1; summed in degree
 * order, so sd agrees with the reference's vertex-order sum to rounding).
 * dist_ac / dist_rel_ac: degree_dist_ac's accumulated log2 distribution and
 * its percentages, bit-identical to the reference: [0] and [1] = vertices
 * of degree 0 and 1, [b] (b >= 2) = vertices with degree in
 * [2^(b-1), 2^b), for 2^(b-1) < max_degree only (as in degree.c, a maximum
 * that is a power of two falls in no bucket).  dist (may be NULL) receives
 * the per-degree counts (degree_dist) of degrees 0 .. min(dist_cap,
 * max_degree + 1) - 1. */
#define TBFS_DEGREE_IN 0
#define TBFS_DEGREE_OUT 1
#define TBFS_DEGREE_UNDIRECTED 2
#define TBFS_DEGREE_BUCKETS 40
typedef struct tbfs_degree_stats {
  int64_t max_degree;
  int64_t argmax;
  int64_t sum;
  double mean;
  double sd;
  int64_t dist_ac[TBFS_DEGREE_BUCKETS];
  double dist_rel_ac[TBFS_DEGREE_BUCKETS];
} tbfs_degree_stats;
tbfs_status tbfs_graph_degree_stats(tbfs_graph *g, int32_t kind, tbfs_degree_stats *out,
                                    int64_t *dist, int64_t dist_cap);

/* Autotuner: picks the single-source engine's shape (max_ept, ctas_per_sm)
 * and then alpha, beta and pull_ratio for g by timing traversals from the k
 * sample roots (device events; the shape over a small grid at opt's
 * direction parameters, then every combination of a grid of those at the
 * chosen shape) and writes them into *opt, leaving its other fields as they
 * are.  With cache_path (a text file; NULL: no cache) the result is stored
 * under a key made of the graph's degree-profile shape, and a later call on
 * a graph with the same key returns the stored values without timing
 * (*from_cache = 1). */
tbfs_status tbfs_autotune(tbfs_graph *g, const int32_t *roots, int32_t k, const char *cache_path,
                          tbfs_options *opt, int32_t *from_cache);

/* The same for tbfs_bfs_batch: picks opt->alpha, the frontier-matrix batch's
 * push/pull threshold, by timing one batch launch of the k (<= 256) roots per
 * candidate (with or without path counts as opt->want_sigma); cached per
 * degree-profile shape and root count. */
tbfs_status tbfs_autotune_batch(tbfs_graph *g, const int32_t *roots, int32_t k,
                                const char *cache_path, tbfs_options *opt, int32_t *from_cache);

/* Betweenness centrality over the given roots: bc[v] = sum over roots s != v
 * of Brandes' dependency delta_s(v) (U. Brandes, J. Math. Sociology 25(2),
 * 2001), unnormalised; on an undirected graph every pair is counted in both
 * directions (divide by 2 for the usual convention when all vertices are
 * roots).  The forward phase is the engine's BFS (S, sigma); the dependency
 * sweep pulls over out-lists level by level in a fixed summation order
 * (below 32 entries in list order; otherwise strided by 32 and combined by
 * a butterfly), with correctly rounded double operations, so results are
 * reproducible bit for bit; the order of out-lists built on the device for
 * a graph without TBFS_GRAPH_SYMMETRIC is not fixed, so there they agree to
 * rounding.  bc (n doubles) is host or device memory per
 * opt->outputs_on_device; *overflow (may be NULL) receives the number of
 * roots whose path counts passed INT64_MAX (their ratios are then inexact). */
tbfs_status tbfs_brandes(tbfs_graph *g, const int32_t *roots, int32_t k, const tbfs_options *opt,
                         double *bc, int32_t *overflow);

/* ---- many graphs, one root each: a packed arena ----
 * No counterpart in the reference.  g graphs in one int32 offset arena:
 * graph i has n[i] vertices and nnz[i] CSC entries; col_ptr holds the g
 * column-pointer arrays one after another (n[i] + 1 entries each, 0-based
 * within the graph) and row_idx the g row-index arrays (nnz[i] each).
 * flags: TBFS_GRAPH_SYMMETRIC when every graph is undirected (in-lists
 * double as out-lists); otherwise out-lists are built.  The arena keeps its
 * vertex numbering.  tbfs_arena_bfs runs one BFS per graph from roots[i]
 * (vertex of graph i), all graphs advancing together in one persistent
 * launch (1024 at a time); S and sigma are packed like the arena (graph i at
 * vertex offset n[0] + ... + n[i-1]) and stats gets g records.  Every
 * traversal is top-down with exact int64 path counts. */
typedef struct tbfs_arena tbfs_arena;
tbfs_status tbfs_arena_create(int32_t g, const int32_t *n, const int64_t *nnz,
                              const int32_t *col_ptr, const int32_t *row_idx,
                              uint32_t flags, tbfs_arena **out);
tbfs_status tbfs_arena_info(const tbfs_arena *a, int32_t *g, int64_t *vertices,
                            int64_t *entries);
tbfs_status tbfs_arena_bfs(tbfs_arena *a, const int32_t *roots, const tbfs_options *opt,
                           int32_t *S, int64_t *sigma, tbfs_stats *stats);
void tbfs_arena_destroy(tbfs_arena *a);

/* ---- serving: a request loop with continuous batching ----
 * No counterpart in the reference.  tbfs_server_create starts a host thread
 * owning a device-memory pool of mem_budget bytes and max_slots (<= 1024)
 * traversal slots on the current device.  tbfs_server_submit queues a query
 * (resident graph g, root) whose results go to the caller's host arrays S[n]
 * and sigma[n] (sigma NULL: depths only), which must stay valid until
 * tbfs_server_wait(ticket) returns.  The loop admits queued queries into free
 * slots while the pool has room (about 48 n bytes per query with path
 * counts, 32 n without), runs one persistent launch that advances every
 * admitted query level by level -- until a query finishes or a new one is
 * submitted, so that results leave and newcomers join at level
 * boundaries -- and retires the finished ones.  Queries on large graphs
 * (2^17 vertices or more) whose last traversal had at most 48 levels run
 * instead, one at a time between those launches, on the single-source
 * direction-optimizing engine (tbfs_bfs on the server's stream); callers
 * must not traverse a served graph themselves while queries on it are
 * pending.  Results equal tbfs_bfs's for the same (graph, root)
 * whatever else is running.  wait returns the query's status, statistics
 * and latency (submit to results in host memory, ms).  The graphs must
 * outlive their queries.  destroy fails queued queries, finishes running
 * ones and stops the thread. */
typedef struct tbfs_server tbfs_server;
tbfs_status tbfs_server_create(int32_t max_slots, int64_t mem_budget, const tbfs_options *opt,
                               tbfs_server **out);
tbfs_status tbfs_server_submit(tbfs_server *s, tbfs_graph *g, int32_t root, int32_t *S,
                               int64_t *sigma, uint64_t *ticket);
tbfs_status tbfs_server_wait(tbfs_server *s, uint64_t ticket, tbfs_stats *stats,
                             double *latency_ms);
tbfs_status tbfs_server_counters(tbfs_server *s, int64_t *launches, int64_t *levels,
                                 int64_t *completed);
/* Where the server's time went (host wall clock, ms, cumulative): its
 * thread in multi-instance launches (enqueue to completion) and in routed
 * single-source queries; its delivery thread copying finished results to
 * the callers' arrays, which overlaps the next launches; the number of
 * routed queries, and the sum over launches of the slots each one ran
 * (divided by launches: mean batch width). */
tbfs_status tbfs_server_time_split(tbfs_server *s, double *launch_ms, double *plain_ms,
                                   double *deliver_ms, int64_t *plain_runs, int64_t *slot_sum);
void tbfs_server_destroy(tbfs_server *s);

/* One BFS that allocates nothing.  No counterpart in the reference: it is
 * for callers that must not have a library call cudaMalloc or cudaFree --
 * code running under a host framework that owns all device memory through
 * its own pool, or a latency-critical loop that cannot take the device-wide
 * synchronisation those calls may cause.  Every pointer is a device pointer
 * the caller owns: the CSC in-lists, optionally separate out-lists
 * (d_out_ptr/d_out_idx; NULL for a symmetric graph), S[n] and sigma[n]
 * (sigma may be NULL for depths only).  Scratch (frontier queues, control
 * block) is a static device array inside the library sized for at most
 * TBFS_NOALLOC_MAX_VERTICES vertices (about 36 MB held on every GPU where
 * the library's device code is loaded, until exit); larger n is rejected
 * with TBFS_ERR_UNSUPPORTED.  The first call on a device looks up that
 * array's device address; since CUDA loads device code lazily, on a device
 * where nothing else of the library ran yet it also commits the 36 MB (a
 * warm-up call belongs before the host framework reserves device memory,
 * and before any stream capture; without the memory the call returns
 * TBFS_ERR_OUT_OF_MEMORY).  All calls share the array: calls whose GPU work
 * overlaps race.  The input is validated on the device each call; the call
 * waits for the traversal to finish on `stream` (NULL = legacy default
 * stream) before it returns; stats->device_ms is left 0. */
#define TBFS_NOALLOC_MAX_VERTICES (1 << 20)
tbfs_status tbfs_bfs_noalloc(const int32_t *d_col_ptr, const int32_t *d_row_idx,
                             const int32_t *d_out_ptr, const int32_t *d_out_idx,
                             int32_t n, int64_t nnz, int32_t root, int32_t mode,
                             int32_t *d_S, int64_t *d_sigma, void *stream,
                             tbfs_stats *stats);

/* Device memory the library freed stays mapped in its pool (up to
 * TBFS_POOL_KEEP_MB, default 8192 MB, per GPU) for the next graph or
 * workspace; this hands all of it back to the CUDA driver now. */
tbfs_status tbfs_release_cached_memory(void);

/* Page-locked host buffers for fast host<->device copies. */
tbfs_status tbfs_host_alloc_pinned(size_t bytes, void **ptr);
void tbfs_host_free_pinned(void *ptr);

const char *tbfs_status_string(tbfs_status s);
/* Detail of the last failure on the calling thread ("" if none). */
const char *tbfs_last_error(void);
int32_t tbfs_version(void);
/* Number of visible CUDA devices (0 on a machine without a GPU). */
int32_t tbfs_device_count(void);

#ifdef __cplusplus
}
#endif
#endif /* TBFS_H */
