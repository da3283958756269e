/*
 * tbfs_internal.h -- types shared by the engine's translation units.
 *
 * HBM layout of one resident graph (n vertices, nnz CSC entries):
 *   cp[n+1], ic[nnz]   int32 CSC: in-lists (column v = sources of edges ->v)
 *   rp[n+1], jr[nnz]   int32 out-lists; aliases cp/ic when the graph is
 *                      symmetric, else the transpose built on the device
 * Per-traversal workspace (reused across calls on the same graph):
 *   q0[n], q1[n]       int32 frontier queues (ping-pong by level parity)
 *   e0[n], e1[n]       int32 out-edge offset of each queue entry (exclusive
 *                      prefix of out-degrees, in queue order)
 *   ctl                control block: per-level counters, barrier words
 * Outputs: S[n] int32 (-1 unreached), sigma[n] uint64 bit patterns of the
 * int64 path counts.
 */
#ifndef TBFS_INTERNAL_H
#define TBFS_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "tbfs.h"

namespace tbfs {

/* Device control block of one traversal; zeroed before every launch. */
struct __align__(128) BfsCtl {
  /* slot d % 3 accumulates the queue of level d+1 ... see bfs_engine.cu */
  unsigned long long qctr[3];
  int status;          /* TBFS_OK or TBFS_ERR_TIMEOUT                     */
  int sigma_overflow;  /* some path count passed INT64_MAX               */
  int levels, td_levels, bu_levels;
  int timeout_level;   /* level + 2 of the barrier that gave up, else 0  */
  long long visited, edges;
  unsigned int pad0[14];
  /* barrier words on their own 128-byte lines */
  unsigned int bar_arrive;
  unsigned int pad1[31];
  unsigned int bar_gen;
  unsigned int pad2[31];
};

struct BfsParams {
  const int *cp, *ic; /* in-lists  */
  const int *rp, *jr; /* out-lists */
  int *S;
  unsigned long long *sigma; /* null: S only */
  int *q0, *q1, *e0, *e1;
  BfsCtl *ctl;
  long long out_edges_total;
  long long timeout_ns;
  int n, root, mode, symmetric;
  float alpha, beta;
  int inject_barrier_skip; /* test hook, 0 = off */
};

/* Launch geometry of the persistent kernel on the current device. */
struct LaunchGeom {
  int grid = 0;
  int block = 0;
};

cudaError_t bfs_launch(const BfsParams &p, const LaunchGeom &g, cudaStream_t s);
cudaError_t bfs_geometry(int device, LaunchGeom *out);

/* graph ingest helpers (graph_ingest.cu) */
cudaError_t validate_csc(const int *cp, const int *ic, int n, long long nnz,
                         int *d_flag, cudaStream_t s);
cudaError_t counting_sort_lists(const int *keys, const int *vals, long long nnz,
                                int n, int *ptr_out, int *idx_out, int *d_flag,
                                cudaStream_t s);
cudaError_t expand_columns(const int *cp, int n, int *col_of_entry, cudaStream_t s);

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
  int *q0 = nullptr, *q1 = nullptr, *e0 = nullptr, *e1 = nullptr;
  tbfs::BfsCtl *ctl = nullptr;
  tbfs::BfsCtl *ctl_host = nullptr; /* pinned mirror */
  int *S_dev = nullptr;
  unsigned long long *sigma_dev = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t last_stream = nullptr;
  tbfs::LaunchGeom geom;
  bool pending = false; /* a traversal was enqueued and not yet collected */
  tbfs_stats last = {};
};

extern "C" void tbfs_set_error(const char *fmt, ...);

#endif
