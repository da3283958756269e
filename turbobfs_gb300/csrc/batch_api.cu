/*
 * batch_api.cu -- tbfs_bfs_batch: many roots on one resident graph through
 * the frontier-matrix engine (batch_engine.cu), 256 roots per launch.
 *
 * Workspace (per graph, allocated on first use, grown when a launch needs
 * wider rows, freed with the graph): seen and three frontier rows of W words
 * per vertex, three frontier queues with their hub sub-queues, the
 * queue-membership bitmap, per-vertex segment arrival counters, and the
 * per-(vertex, root) depth and path-count rows of 32 W entries.  For
 * RMAT scale 20 with 256 roots (W = 8) that is about 3.3 GB, plus a staging
 * copy of the results when the caller wants them in host memory.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "tbfs.h"
#include "tbfs_internal.h"

namespace tbfs {

struct BatchWS {
  int n = 0, W = 0;
  bool sigma = false;
  unsigned *seen = nullptr, *F = nullptr, *touched = nullptr, *seg_arrive = nullptr;
  int *q = nullptr, *hq = nullptr;
  unsigned *e = nullptr, *he = nullptr;
  int *S_int = nullptr;
  unsigned long long *sig_int = nullptr;
  int *hubs = nullptr, *hub_seg = nullptr;
  int nhub = 0, hub_segs = 0, seg_len = 0;
  BatchCtl *ctl = nullptr, *ctl_host = nullptr;
  int *roots_dev = nullptr, *roots_host = nullptr;
  /* per-root statistics: visited[256], edges[256] (u64), max depth[256] (int) */
  unsigned long long *rst = nullptr, *rst_host = nullptr;
  int *S_stage = nullptr;
  unsigned long long *sig_stage = nullptr;
  size_t stage_entries = 0;
  bool stage_sigma = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  long long *trace_dev = nullptr;
  int trace_cap = 0;
};

tbfs_status fail(cudaError_t e, const char *what) {
  tbfs_set_error("tbfs_bfs_batch: %s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
}

namespace {

constexpr size_t kStatBytes = (size_t)kBatchMaxRoots * (2 * sizeof(unsigned long long) + sizeof(int));

void free_rows(BatchWS *w) {
  tbfs::dev_free(w->seen);
  tbfs::dev_free(w->F);
  tbfs::dev_free(w->S_int);
  tbfs::dev_free(w->sig_int);
  tbfs::dev_free(w->hubs);
  tbfs::dev_free(w->hub_seg);
  w->seen = w->F = nullptr;
  w->S_int = nullptr;
  w->sig_int = nullptr;
  w->hubs = w->hub_seg = nullptr;
  w->W = 0;
  w->sigma = false;
}

#define TRY(call, what)                               \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return tbfs::fail(e_, what); \
  } while (0)

/* the workspace for rows of W words (and path counts if sigma) */
tbfs_status ensure_ws(tbfs_graph *g, int W, bool sigma, cudaStream_t s) {
  if (!g->batch) g->batch = new BatchWS();
  BatchWS *w = g->batch;
  const size_t n = (size_t)g->n;
  if (!w->ctl) {
    w->n = g->n;
    TRY(tbfs::dev_alloc(&w->touched, ((n + 31) / 32) * sizeof(unsigned)), "alloc");
    TRY(tbfs::dev_alloc(&w->seg_arrive, n * sizeof(unsigned)), "alloc");
    TRY(tbfs::dev_alloc(&w->q, 3 * n * sizeof(int)), "alloc");
    TRY(tbfs::dev_alloc(&w->e, 3 * n * sizeof(unsigned)), "alloc");
    TRY(tbfs::dev_alloc(&w->hq, 3 * n * sizeof(int)), "alloc");
    TRY(tbfs::dev_alloc(&w->he, 3 * n * sizeof(unsigned)), "alloc");
    TRY(tbfs::dev_alloc(&w->roots_dev, kBatchMaxRoots * sizeof(int)), "alloc");
    TRY(cudaMallocHost(&w->roots_host, kBatchMaxRoots * sizeof(int)), "alloc");
    TRY(tbfs::dev_alloc(&w->rst, kStatBytes), "alloc");
    TRY(cudaMallocHost(&w->rst_host, kStatBytes), "alloc");
    TRY(tbfs::dev_alloc(&w->ctl, sizeof(BatchCtl)), "alloc");
    TRY(cudaMallocHost(&w->ctl_host, sizeof(BatchCtl)), "alloc");
    TRY(cudaEventCreate(&w->ev0), "event");
    TRY(cudaEventCreate(&w->ev1), "event");
  }
  if (w->W != W || (sigma && !w->sigma)) {
    const bool keep_sigma = sigma || (w->sigma && w->W == W);
    free_rows(w);
    const size_t rs = 32 * (size_t)W;
    TRY(tbfs::dev_alloc(&w->seen, n * W * sizeof(unsigned)), "alloc rows");
    TRY(tbfs::dev_alloc(&w->F, 3 * n * W * sizeof(unsigned)), "alloc rows");
    TRY(tbfs::dev_alloc(&w->S_int, n * rs * sizeof(int)), "alloc depth rows");
    if (keep_sigma) TRY(tbfs::dev_alloc(&w->sig_int, n * rs * sizeof(unsigned long long)), "alloc count rows");
#ifndef TBFS_BATCH_SEG
#define TBFS_BATCH_SEG 128
#endif
    w->seg_len = TBFS_BATCH_SEG * W; /* a hub segment: about one work item of the pull */
    TRY(batch_hubs(g->cp, g->n, w->seg_len, &w->hubs, &w->hub_seg, &w->nhub, &w->hub_segs, s),
        "hub list");
    w->W = W;
    w->sigma = keep_sigma;
  }
  return TBFS_OK;
}

tbfs_status ensure_stage(BatchWS *w, size_t entries, bool sigma) {
  if (w->stage_entries >= entries && (!sigma || w->stage_sigma)) return TBFS_OK;
  tbfs::dev_free(w->S_stage);
  tbfs::dev_free(w->sig_stage);
  w->S_stage = nullptr;
  w->sig_stage = nullptr;
  w->stage_entries = 0;
  w->stage_sigma = false;
  TRY(tbfs::dev_alloc(&w->S_stage, entries * sizeof(int)), "alloc staging");
  if (sigma) TRY(tbfs::dev_alloc(&w->sig_stage, entries * sizeof(unsigned long long)), "alloc staging");
  w->stage_entries = entries;
  w->stage_sigma = sigma;
  return TBFS_OK;
}

int width_for(int k) { return k <= 32 ? 1 : k <= 64 ? 2 : k <= 128 ? 4 : 8; }

}  // namespace

void batch_ws_free(BatchWS *w) {
  if (!w) return;
  free_rows(w);
  tbfs::dev_free(w->touched);
  tbfs::dev_free(w->seg_arrive);
  tbfs::dev_free(w->q);
  tbfs::dev_free(w->e);
  tbfs::dev_free(w->hq);
  tbfs::dev_free(w->he);
  tbfs::dev_free(w->roots_dev);
  tbfs::dev_free(w->rst);
  tbfs::dev_free(w->ctl);
  tbfs::dev_free(w->S_stage);
  tbfs::dev_free(w->sig_stage);
  tbfs::dev_free(w->trace_dev);
  if (w->roots_host) cudaFreeHost(w->roots_host);
  if (w->rst_host) cudaFreeHost(w->rst_host);
  if (w->ctl_host) cudaFreeHost(w->ctl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

}  // namespace tbfs

using tbfs::BatchWS;

extern "C" tbfs_status tbfs_bfs_batch(tbfs_graph *g, const int32_t *roots, int32_t k,
                                      const tbfs_options *opt, int32_t layout, int32_t *S,
                                      int64_t *sigma, tbfs_stats *stats) {
  tbfs_options o;
  tbfs_options_init(&o);
  if (opt) o = *opt;
  if (!g || k < 0 || (k > 0 && !roots)) {
    tbfs_set_error("tbfs_bfs_batch: null graph or roots, or k < 0");
    return TBFS_ERR_INVALID_ARG;
  }
  if (layout != TBFS_LAYOUT_ROOT_MAJOR && layout != TBFS_LAYOUT_VERTEX_MAJOR) {
    tbfs_set_error("tbfs_bfs_batch: layout must be TBFS_LAYOUT_ROOT_MAJOR or _VERTEX_MAJOR");
    return TBFS_ERR_INVALID_ARG;
  }
  if (k == 0) return TBFS_OK;
  if (!S || (o.want_sigma && !sigma)) {
    tbfs_set_error("tbfs_bfs_batch: null S output, or want_sigma set and sigma null");
    return TBFS_ERR_INVALID_ARG;
  }
  if (o.mode < TBFS_MODE_AUTO || o.mode > TBFS_MODE_BOTTOM_UP || !(o.alpha > 0.0f)) {
    tbfs_set_error("tbfs_bfs_batch: bad mode or alpha");
    return TBFS_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) {
      tbfs_set_error("tbfs_bfs_batch: root %d (index %d) outside [0, n)", roots[i], i);
      return TBFS_ERR_INVALID_ARG;
    }
  TRY(cudaSetDevice(g->device), "cudaSetDevice");
  cudaStream_t s = (cudaStream_t)o.stream;
  const bool want_sigma = o.want_sigma != 0;
  const size_t n = (size_t)g->n;
  const long long timeout = o.timeout_ns > 0 ? o.timeout_ns : 4000000000LL;

  for (int32_t r0 = 0; r0 < k; r0 += tbfs::kBatchMaxRoots) {
    const int kg = std::min<int32_t>(tbfs::kBatchMaxRoots, k - r0);
    const int W = tbfs::width_for(kg);
    tbfs_status st = tbfs::ensure_ws(g, W, want_sigma, s);
    if (st != TBFS_OK) return st;
    BatchWS *w = g->batch;
    /* path counts in 32 bits first: half the bytes per hit; a launch that
     * meets a count needing more is redone with 64-bit counts */
    int sigmode = want_sigma ? 2 : 0;
    tbfs::LaunchGeom geom;
    TRY(tbfs::batch_geometry(g->device, W, sigmode, &geom), "launch geometry");

    memcpy(w->roots_host, roots + r0, (size_t)kg * sizeof(int));
    TRY(cudaMemcpyAsync(w->roots_dev, w->roots_host, (size_t)kg * sizeof(int),
                        cudaMemcpyHostToDevice, s),
        "roots upload");
    TRY(cudaMemsetAsync(w->ctl, 0, sizeof(tbfs::BatchCtl), s), "clear control block");
    TRY(cudaMemsetAsync(w->rst, 0, 2 * tbfs::kBatchMaxRoots * sizeof(unsigned long long), s),
        "clear stats");
    TRY(cudaMemsetAsync(w->rst + 2 * tbfs::kBatchMaxRoots, 0xff, tbfs::kBatchMaxRoots * sizeof(int),
                        s),
        "clear stats");

    tbfs::BatchParams p;
    memset(&p, 0, sizeof(p));
    p.cp = g->cp;
    p.ic = g->ic;
    p.rp = g->rp;
    p.jr = g->jr;
    p.n = g->n;
    p.nnz_in = g->nnz;
    p.k = kg;
    p.roots = w->roots_dev;
    p.inv = g->inv;
    p.seen = w->seen;
    for (int b = 0; b < 3; ++b) {
      p.F[b] = w->F + (size_t)b * n * W;
      p.q[b] = w->q + (size_t)b * n;
      p.e[b] = w->e + (size_t)b * n;
      p.hq[b] = w->hq + (size_t)b * n;
      p.he[b] = w->he + (size_t)b * n;
    }
    p.touched = w->touched;
    p.seg_arrive = w->seg_arrive;
    p.S_int = w->S_int;
    p.sig_int = want_sigma ? w->sig_int : nullptr;
    p.hubs = w->hubs;
    p.hub_seg = w->hub_seg;
    p.nhub = w->nhub;
    p.hub_segs = w->hub_segs;
    p.seg_len = w->seg_len;
    p.ctl = w->ctl;
    p.timeout_ns = timeout;
    p.alpha = o.alpha;
    p.mode = o.mode;
    /* level trace of the first launch (roots 0..255) */
    const bool tracing = r0 == 0 && o.level_trace != nullptr && o.level_trace_cap >= 2;
    if (tracing) {
      if (w->trace_cap < o.level_trace_cap) {
        tbfs::dev_free(w->trace_dev);
        w->trace_dev = nullptr;
        w->trace_cap = 0;
        TRY(tbfs::dev_alloc(&w->trace_dev, (size_t)o.level_trace_cap * 4 * sizeof(long long)), "alloc trace");
        w->trace_cap = o.level_trace_cap;
      }
      TRY(cudaMemsetAsync(w->trace_dev, 0, (size_t)o.level_trace_cap * 4 * sizeof(long long), s),
          "clear trace");
      p.trace = w->trace_dev;
      p.trace_cap = o.level_trace_cap;
    }
    /* root r lives at bit 8 (c % G) + 2 (c / G) + (r & 1) of a row, c = r / 2,
     * G = 4 W (lane-major order, see batch_engine.cu) */
    for (int i = 0; i < 8; ++i) p.valid[i] = 0u;
    for (int r = 0; r < kg; ++r) {
      const int c = r >> 1, G = 4 * W;
      const int b = 8 * (c % G) + 2 * (c / G) + (r & 1);
      p.valid[b >> 5] |= 1u << (b & 31);
    }

    /* where the results go */
    int *S_out;
    unsigned long long *sig_out = nullptr;
    long long ldo;
    if (o.outputs_on_device) {
      if (layout == TBFS_LAYOUT_ROOT_MAJOR) {
        S_out = S + (size_t)r0 * n;
        if (want_sigma) sig_out = reinterpret_cast<unsigned long long *>(sigma) + (size_t)r0 * n;
        ldo = (long long)n;
      } else {
        S_out = S + r0;
        if (want_sigma) sig_out = reinterpret_cast<unsigned long long *>(sigma) + r0;
        ldo = k;
      }
    } else {
      if ((st = tbfs::ensure_stage(w, (size_t)kg * n, want_sigma)) != TBFS_OK) return st;
      S_out = w->S_stage;
      sig_out = want_sigma ? w->sig_stage : nullptr;
      ldo = layout == TBFS_LAYOUT_ROOT_MAJOR ? (long long)n : kg;
    }
    tbfs::BatchOutParams op;
    op.n = g->n;
    op.k = kg;
    op.W = W;
    op.layout = layout;
    op.ldo = ldo;
    op.inv = g->inv;
    op.rp = g->rp;
    op.seen = w->seen;
    op.S_int = w->S_int;
    op.sig_int = want_sigma ? w->sig_int : nullptr;
    op.S_out = S_out;
    op.sig_out = sig_out;
    op.r_visited = w->rst;
    op.r_edges = w->rst + tbfs::kBatchMaxRoots;
    op.r_maxd = reinterpret_cast<int *>(w->rst + 2 * tbfs::kBatchMaxRoots);

    TRY(cudaEventRecord(w->ev0, s), "event");
    TRY(tbfs::batch_launch(p, W, sigmode, geom, s), "batch launch");
    if (sigmode == 2) {
      TRY(cudaMemcpyAsync(w->ctl_host, w->ctl, sizeof(tbfs::BatchCtl), cudaMemcpyDeviceToHost, s),
          "read control block");
      TRY(cudaStreamSynchronize(s), "batch traversal");
      if (w->ctl_host->wide && w->ctl_host->status == 0) {
        sigmode = 1;
        TRY(tbfs::batch_geometry(g->device, W, sigmode, &geom), "launch geometry");
        TRY(cudaMemsetAsync(w->ctl, 0, sizeof(tbfs::BatchCtl), s), "clear control block");
        TRY(tbfs::batch_launch(p, W, sigmode, geom, s), "batch launch");
      }
    }
    TRY(tbfs::batch_output(op, sigmode, s), "batch results");
    TRY(cudaEventRecord(w->ev1, s), "event");
    TRY(cudaMemcpyAsync(w->ctl_host, w->ctl, sizeof(tbfs::BatchCtl), cudaMemcpyDeviceToHost, s),
        "read control block");
    TRY(cudaMemcpyAsync(w->rst_host, w->rst, tbfs::kStatBytes, cudaMemcpyDeviceToHost, s),
        "read stats");
    if (tracing)
      TRY(cudaMemcpyAsync(o.level_trace, w->trace_dev, (size_t)o.level_trace_cap * 4 * sizeof(long long),
                          cudaMemcpyDeviceToHost, s),
          "read trace");
    if (!o.outputs_on_device) {
      if (layout == TBFS_LAYOUT_ROOT_MAJOR) {
        TRY(cudaMemcpyAsync(S + (size_t)r0 * n, S_out, (size_t)kg * n * sizeof(int),
                            cudaMemcpyDeviceToHost, s),
            "copy S");
        if (want_sigma)
          TRY(cudaMemcpyAsync(sigma + (size_t)r0 * n, sig_out, (size_t)kg * n * sizeof(int64_t),
                              cudaMemcpyDeviceToHost, s),
              "copy sigma");
      } else {
        TRY(cudaMemcpy2DAsync(S + r0, (size_t)k * sizeof(int), S_out, (size_t)kg * sizeof(int),
                              (size_t)kg * sizeof(int), n, cudaMemcpyDeviceToHost, s),
            "copy S");
        if (want_sigma)
          TRY(cudaMemcpy2DAsync(sigma + r0, (size_t)k * sizeof(int64_t), sig_out,
                                (size_t)kg * sizeof(int64_t), (size_t)kg * sizeof(int64_t), n,
                                cudaMemcpyDeviceToHost, s),
              "copy sigma");
      }
    }
    TRY(cudaStreamSynchronize(s), "batch traversal");
    const tbfs::BatchCtl &c = *w->ctl_host;
    if (c.status != 0) {
      tbfs_set_error("tbfs_bfs_batch: grid barrier wait exceeded its budget (level %d)",
                     c.timeout_level - 2);
      return TBFS_ERR_TIMEOUT;
    }
    float ms = 0.0f;
    TRY(cudaEventElapsedTime(&ms, w->ev0, w->ev1), "event time");
    if (stats) {
      const unsigned long long *vis = w->rst_host;
      const unsigned long long *edg = w->rst_host + tbfs::kBatchMaxRoots;
      const int *mdep = reinterpret_cast<const int *>(w->rst_host + 2 * tbfs::kBatchMaxRoots);
      for (int r = 0; r < kg; ++r) {
        tbfs_stats &t = stats[r0 + r];
        memset(&t, 0, sizeof(t));
        t.levels = mdep[r] + 1;
        t.td_levels = c.push_levels;
        t.bu_levels = c.pull_levels;
        t.sigma_overflow = (int32_t)((c.ovf[r >> 5] >> (r & 31)) & 1u);
        t.visited = (int64_t)vis[r];
        t.edges = (int64_t)edg[r];
        t.device_ms = ms;
      }
    }
  }
  return TBFS_OK;
}
