/*
 * api.cu -- the C ABI: resident graphs, single and repeated traversals, and
 * the drop-in replacements for the reference's GPU entry points.
 */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <random>
#include <vector>

#include "tbfs.h"
#include "tbfs_compat.h"
#include "tbfs_graphgen.h"
#include "tbfs_internal.h"

using tbfs::BfsCtl;
using tbfs::BfsParams;

/* ------------------------------------------------------------- errors */

static thread_local char g_err[512];

extern "C" void tbfs_set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

extern "C" const char *tbfs_last_error(void) { return g_err; }

static tbfs_status cuda_fail(cudaError_t e, const char *what, int line) {
  tbfs_set_error("%s: %s (api.cu:%d)", what, cudaGetErrorString(e), line);
  return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
}

#define CUDA_TRY(call)                                          \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call, __LINE__); \
  } while (0)

static tbfs_status invalid(const char *msg) {
  tbfs_set_error("%s", msg);
  return TBFS_ERR_INVALID_ARG;
}

extern "C" const char *tbfs_status_string(tbfs_status s) {
  switch (s) {
    case TBFS_OK: return "ok";
    case TBFS_ERR_INVALID_ARG: return "invalid argument";
    case TBFS_ERR_CUDA: return "CUDA error";
    case TBFS_ERR_OUT_OF_MEMORY: return "out of memory";
    case TBFS_ERR_TIMEOUT: return "grid barrier timeout";
    case TBFS_ERR_NO_DEVICE: return "no CUDA device";
    case TBFS_ERR_IO: return "I/O error";
    case TBFS_ERR_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

extern "C" int32_t tbfs_version(void) { return TBFS_VERSION; }

extern "C" int32_t tbfs_device_count(void) {
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return c;
}

extern "C" void tbfs_options_init(tbfs_options *opt) {
  if (!opt) return;
  memset(opt, 0, sizeof(*opt));
  opt->mode = TBFS_MODE_AUTO;
  opt->want_sigma = 1;
  opt->alpha = 15.0f;
  opt->beta = 2.0f;
  opt->pull_ratio = 1.0f;
}

extern "C" tbfs_status tbfs_host_alloc_pinned(size_t bytes, void **ptr) {
  if (!ptr) return invalid("tbfs_host_alloc_pinned: null out pointer");
  *ptr = nullptr;
  CUDA_TRY(cudaMallocHost(ptr, bytes ? bytes : 1));
  return TBFS_OK;
}

extern "C" void tbfs_host_free_pinned(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}

/* ------------------------------------------------------------- graphs */

static void graph_free(tbfs_graph *g) {
  if (!g) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(g->device);
  if (g->separate_out) {
    tbfs::dev_free(g->rp);
    tbfs::dev_free(g->jr);
  }
  tbfs::dev_free(g->cp);
  tbfs::dev_free(g->ic);
  tbfs::dev_free(g->queues);
  tbfs::dev_free(g->hot); /* bitmaps, S_work, sigma_work */
  tbfs::dev_free(g->inv);
  tbfs::dev_free(g->perm);
  tbfs::dev_free(g->ctl);
  tbfs::dev_free(g->S_dev);
  tbfs::dev_free(g->sigma_dev);
  tbfs::dev_free(g->S_dev2);
  tbfs::dev_free(g->sigma_dev2);
  if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
  tbfs::dev_free(g->trace_dev);
  if (g->ctl_host) cudaFreeHost(g->ctl_host);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  tbfs::dev_free(g->many_ctl);
  if (g->many_ctl_host) cudaFreeHost(g->many_ctl_host);
  for (auto x : g->many_ev) cudaEventDestroy(x);
  for (auto x : g->many_sync) cudaEventDestroy(x);
  tbfs::batch_ws_free(g->batch);
  cudaSetDevice(cur);
  delete g;
}

extern "C" void tbfs_graph_destroy(tbfs_graph *g) { graph_free(g); }

static tbfs_status need_device() {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess || c == 0) {
    cudaGetLastError();
    tbfs_set_error("no CUDA device visible");
    return TBFS_ERR_NO_DEVICE;
  }
  return TBFS_OK;
}

/* allocations shared by both constructors, after cp/ic/rp/jr are set */
static tbfs_status graph_finish(tbfs_graph *g) {
  const size_t n = (size_t)g->n;
  CUDA_TRY(tbfs::dev_alloc(&g->queues, 9 * n * sizeof(int)));
  /* the arrays the traversal gathers from at random -- path counts, depths,
   * frontier bitmaps -- in one block */
  const size_t sig_b = g->inv ? n * sizeof(unsigned long long) : 0;
  const size_t S_b = g->inv ? (n * sizeof(int) + 255) / 256 * 256 : 0;
  const size_t bm_b = 4 * ((n + 31) / 32) * sizeof(unsigned);
  CUDA_TRY(tbfs::dev_alloc(&g->hot, sig_b + S_b + bm_b));
  if (g->inv) {
    g->sigma_work = reinterpret_cast<unsigned long long *>(g->hot);
    g->S_work = reinterpret_cast<int *>(g->hot + sig_b);
  }
  g->bitmaps = reinterpret_cast<unsigned *>(g->hot + sig_b + S_b);
  CUDA_TRY(tbfs::dev_alloc(&g->ctl, sizeof(BfsCtl)));
  CUDA_TRY(cudaMallocHost(&g->ctl_host, sizeof(BfsCtl)));
  memset(g->ctl_host, 0, sizeof(BfsCtl));
  CUDA_TRY(cudaEventCreate(&g->ev0));
  CUDA_TRY(cudaEventCreate(&g->ev1));
  CUDA_TRY(tbfs::bfs_geometry(g->device, &g->geom));
  g->out_edges_total = g->nnz;
  {
    int64_t hist[40], maxd = 0;
    tbfs_status st = tbfs_graph_degree_profile(g, hist, &maxd, nullptr);
    if (st != TBFS_OK) return st;
    int b = 0;
    while (b < 63 && (1ll << b) <= maxd) ++b; /* maxd < 2^b */
    g->deg_bits = b;
    int max_out = (int)maxd;
    if (g->separate_out) {
      cudaError_t e = tbfs::longest_list(g->rp, g->n, &max_out);
      if (e != cudaSuccess) return cuda_fail(e, "out-degree bound", __LINE__);
    }
    g->short_lists = max_out <= tbfs::kShortList;
  }
  return TBFS_OK;
}

static tbfs_status read_flag(const int *d_flag, cudaStream_t s, int *flag) {
  CUDA_TRY(cudaMemcpyAsync(flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return TBFS_OK;
}

static tbfs_status build_csc(tbfs_graph *g, const int32_t *col_ptr, const int32_t *row_idx,
                             int *d_flag) {
  const size_t n = (size_t)g->n, nnz = (size_t)g->nnz;
  const cudaMemcpyKind kind = (g->flags & TBFS_GRAPH_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice
                                                                  : cudaMemcpyHostToDevice;
  CUDA_TRY(tbfs::dev_alloc(&g->cp, (n + 1) * sizeof(int)));
  CUDA_TRY(tbfs::dev_alloc(&g->ic, (nnz ? nnz : 1) * sizeof(int)));
  CUDA_TRY(cudaMemcpy(g->cp, col_ptr, (n + 1) * sizeof(int), kind));
  if (nnz) CUDA_TRY(cudaMemcpy(g->ic, row_idx, nnz * sizeof(int), kind));
  CUDA_TRY(cudaMemset(d_flag, 0, sizeof(int)));
  CUDA_TRY(tbfs::validate_csc(g->cp, g->ic, g->n, g->nnz, d_flag, 0));
  int flag = 0;
  tbfs_status st = read_flag(d_flag, 0, &flag);
  if (st != TBFS_OK) return st;
  if (flag & 1) return invalid("col_ptr must start at 0, be nondecreasing and end at nnz");
  if (flag & 2) return invalid("row index outside [0, n)");
  return TBFS_OK;
}

/* After the validated in-lists (cp, ic) are on the device: regroup the
 * vertices by degree unless the caller asked to keep the order, then alias
 * (symmetric) or build the out-lists as the transpose. */
static tbfs_status finish_lists(tbfs_graph *g, int *d_flag) {
  const size_t n = (size_t)g->n, nnz = (size_t)g->nnz;
  if (!(g->flags & TBFS_GRAPH_KEEP_ORDER) && nnz > 0) {
    int *perm = nullptr, *inv = nullptr, *cp2 = nullptr, *ic2 = nullptr;
    bool identity = true;
    cudaError_t e = tbfs::dev_alloc(&perm, n * sizeof(int));
    if (e == cudaSuccess) e = tbfs::dev_alloc(&inv, n * sizeof(int));
    if (e == cudaSuccess) e = tbfs::dev_alloc(&cp2, (n + 1) * sizeof(int));
    if (e == cudaSuccess) e = tbfs::dev_alloc(&ic2, nnz * sizeof(int));
    if (e == cudaSuccess)
      e = tbfs::degree_group_relabel(g->cp, g->ic, g->n, g->nnz, perm, inv, cp2, ic2, &identity,
                                     0);
    if (e != cudaSuccess || identity) {
      tbfs::dev_free(perm);
      tbfs::dev_free(inv);
      tbfs::dev_free(cp2);
      tbfs::dev_free(ic2);
      if (e != cudaSuccess) return cuda_fail(e, "degree grouping", __LINE__);
    } else {
      tbfs::dev_free(g->cp);
      tbfs::dev_free(g->ic);
      g->cp = cp2;
      g->ic = ic2;
      g->inv = inv;
      g->perm = perm;
    }
  }
  bool symmetric = (g->flags & TBFS_GRAPH_SYMMETRIC) != 0;
  g->declared_symmetric = symmetric;
  if (!symmetric && nnz > 0) {
    /* no promise from the caller: a CSC that equals its transpose needs no
     * out-lists of its own (fresh random keys each time) */
    static std::atomic<unsigned long long> calls{0};
    const unsigned long long salt =
        (unsigned long long)std::chrono::steady_clock::now().time_since_epoch().count() ^
        (0x9e3779b97f4a7c15ull * ++calls) ^ (unsigned long long)(uintptr_t)g;
    std::random_device rd;
    const unsigned long long k1 = ((unsigned long long)rd() << 32 | rd()) ^ salt;
    const unsigned long long k2 = ((unsigned long long)rd() << 32 | rd()) ^ (salt * 31);
    cudaError_t e = tbfs::symmetric_check(g->cp, g->ic, g->n, g->nnz, k1, k2, &symmetric, 0);
    if (e != cudaSuccess) return cuda_fail(e, "symmetry check", __LINE__);
  }
  if (symmetric) {
    g->rp = g->cp;
    g->jr = g->ic;
    g->flags |= TBFS_GRAPH_SYMMETRIC; /* reported by tbfs_graph_info */
    return TBFS_OK;
  }
  /* out-lists = transpose: key = row id, value = column id */
  int *col = nullptr;
  CUDA_TRY(tbfs::dev_alloc(&col, (nnz ? nnz : 1) * sizeof(int)));
  g->separate_out = true;
  cudaError_t e = tbfs::dev_alloc(&g->rp, (n + 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&g->jr, (nnz ? nnz : 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::expand_columns(g->cp, g->n, col, 0);
  if (e == cudaSuccess)
    e = tbfs::counting_sort_lists(g->ic, col, g->nnz, g->n, g->rp, g->jr, d_flag, 0);
  tbfs::dev_free(col);
  if (e != cudaSuccess) return cuda_fail(e, "transpose", __LINE__);
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_graph_create_csc(const int32_t *col_ptr, const int32_t *row_idx,
                                             int32_t n, int64_t nnz, uint32_t flags,
                                             tbfs_graph **out) {
  if (!out) return invalid("tbfs_graph_create_csc: null out pointer");
  *out = nullptr;
  if (n < 1 || nnz < 0 || nnz > INT32_MAX || !col_ptr || (nnz > 0 && !row_idx))
    return invalid("tbfs_graph_create_csc: need n >= 1, 0 <= nnz <= INT32_MAX, arrays");
  tbfs_status st = need_device();
  if (st != TBFS_OK) return st;
  tbfs_graph *g = new tbfs_graph();
  cudaGetDevice(&g->device);
  g->n = n;
  g->nnz = nnz;
  g->flags = flags;
  int *d_flag = nullptr;
  cudaError_t e = tbfs::dev_alloc(&d_flag, sizeof(int));
  if (e != cudaSuccess) {
    graph_free(g);
    return cuda_fail(e, "tbfs::dev_alloc(flag)", __LINE__);
  }
  st = build_csc(g, col_ptr, row_idx, d_flag);
  if (st == TBFS_OK) st = finish_lists(g, d_flag);
  tbfs::dev_free(d_flag);
  if (st == TBFS_OK) st = graph_finish(g);
  if (st != TBFS_OK) {
    graph_free(g);
    return st;
  }
  *out = g;
  return TBFS_OK;
}

static tbfs_status build_cooc(tbfs_graph *g, const int32_t *row, const int32_t *col,
                              int *d_flag) {
  const size_t n = (size_t)g->n, nnz = (size_t)g->nnz;
  const cudaMemcpyKind kind = (g->flags & TBFS_GRAPH_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice
                                                                  : cudaMemcpyHostToDevice;
  int *dr = nullptr, *dc = nullptr;
  cudaError_t e = tbfs::dev_alloc(&dr, (nnz ? nnz : 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dc, (nnz ? nnz : 1) * sizeof(int));
  if (e == cudaSuccess && nnz) e = cudaMemcpy(dr, row, nnz * sizeof(int), kind);
  if (e == cudaSuccess && nnz) e = cudaMemcpy(dc, col, nnz * sizeof(int), kind);
  if (e == cudaSuccess) e = cudaMemset(d_flag, 0, sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&g->cp, (n + 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&g->ic, (nnz ? nnz : 1) * sizeof(int));
  /* in-lists: key = column (target), value = row (source) */
  if (e == cudaSuccess)
    e = tbfs::counting_sort_lists(dc, dr, g->nnz, g->n, g->cp, g->ic, d_flag, 0);
  tbfs::dev_free(dr);
  tbfs::dev_free(dc);
  if (e != cudaSuccess) return cuda_fail(e, "COOC ingest", __LINE__);
  int flag = 0;
  tbfs_status st = read_flag(d_flag, 0, &flag);
  if (st != TBFS_OK) return st;
  if (flag) return invalid("COOC entry outside [0, n)");
  return finish_lists(g, d_flag);
}

extern "C" tbfs_status tbfs_graph_create_cooc(const int32_t *row, const int32_t *col,
                                              int32_t n, int64_t nnz, uint32_t flags,
                                              tbfs_graph **out) {
  if (!out) return invalid("tbfs_graph_create_cooc: null out pointer");
  *out = nullptr;
  if (n < 1 || nnz < 0 || nnz > INT32_MAX || (nnz > 0 && (!row || !col)))
    return invalid("tbfs_graph_create_cooc: need n >= 1, 0 <= nnz <= INT32_MAX, arrays");
  tbfs_status st = need_device();
  if (st != TBFS_OK) return st;
  tbfs_graph *g = new tbfs_graph();
  cudaGetDevice(&g->device);
  g->n = n;
  g->nnz = nnz;
  g->flags = flags;
  int *d_flag = nullptr;
  cudaError_t e = tbfs::dev_alloc(&d_flag, sizeof(int));
  if (e != cudaSuccess) {
    graph_free(g);
    return cuda_fail(e, "tbfs::dev_alloc(flag)", __LINE__);
  }
  st = build_cooc(g, row, col, d_flag);
  tbfs::dev_free(d_flag);
  if (st == TBFS_OK) st = graph_finish(g);
  if (st != TBFS_OK) {
    graph_free(g);
    return st;
  }
  *out = g;
  return TBFS_OK;
}

/* ------------------------------------------- device-built graphs */

/* A graph from an edge list already on the device: CSC built there with the
 * host builder's construction, then the usual regrouping / out-lists. */
static tbfs_status graph_from_device_edges(const int *d_src, const int *d_dst, int32_t n,
                                           int64_t m, uint32_t build_flags, uint32_t graph_flags,
                                           tbfs_graph **out) {
  tbfs_graph *g = new tbfs_graph();
  cudaGetDevice(&g->device);
  g->n = n;
  g->flags = graph_flags & ~TBFS_GRAPH_DEVICE_PTRS;
  if (build_flags & TBFS_BUILD_SYMMETRIZE) g->flags |= TBFS_GRAPH_SYMMETRIC;
  long long nnz = 0;
  int bad = 0;
  cudaError_t e = tbfs::csc_from_edges_device(d_src, d_dst, m, n, build_flags, &g->cp, &g->ic,
                                              &nnz, &bad, 0);
  if (e != cudaSuccess) {
    graph_free(g);
    if (e == cudaErrorInvalidValue) {
      tbfs_set_error("edge list: more than INT32_MAX list entries");
      return TBFS_ERR_UNSUPPORTED;
    }
    return cuda_fail(e, "edge list -> CSC on the device", __LINE__);
  }
  if (bad) {
    graph_free(g);
    return invalid("edge list: endpoint outside [0, n)");
  }
  if (nnz > INT32_MAX) {
    graph_free(g);
    tbfs_set_error("edge list: %lld CSC entries exceed int32", nnz);
    return TBFS_ERR_UNSUPPORTED;
  }
  g->nnz = nnz;
  int *d_flag = nullptr;
  e = tbfs::dev_alloc(&d_flag, sizeof(int));
  if (e != cudaSuccess) {
    graph_free(g);
    return cuda_fail(e, "tbfs::dev_alloc(flag)", __LINE__);
  }
  cudaMemset(d_flag, 0, sizeof(int));
  tbfs_status st = finish_lists(g, d_flag);
  tbfs::dev_free(d_flag);
  if (st == TBFS_OK) st = graph_finish(g);
  if (st != TBFS_OK) {
    graph_free(g);
    return st;
  }
  *out = g;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_graph_create_edges(const int32_t *src, const int32_t *dst,
                                               int32_t n, int64_t m, uint32_t build_flags,
                                               uint32_t graph_flags, tbfs_graph **out) {
  if (!out) return invalid("tbfs_graph_create_edges: null out pointer");
  *out = nullptr;
  if (n < 1 || m < 0 || (m > 0 && (!src || !dst)))
    return invalid("tbfs_graph_create_edges: need n >= 1, m >= 0, arrays");
  if (m > ((build_flags & TBFS_BUILD_SYMMETRIZE) ? INT32_MAX / 2 : INT32_MAX)) {
    tbfs_set_error("tbfs_graph_create_edges: too many edges for int32 lists");
    return TBFS_ERR_UNSUPPORTED;
  }
  tbfs_status st = need_device();
  if (st != TBFS_OK) return st;
  if (graph_flags & TBFS_GRAPH_DEVICE_PTRS)
    return graph_from_device_edges(src, dst, n, m, build_flags, graph_flags, out);
  int *ds = nullptr, *dd = nullptr;
  const size_t bytes = (size_t)(m > 0 ? m : 1) * sizeof(int);
  cudaError_t e = tbfs::dev_alloc(&ds, bytes);
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dd, bytes);
  if (e == cudaSuccess && m > 0) e = cudaMemcpy(ds, src, (size_t)m * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && m > 0) e = cudaMemcpy(dd, dst, (size_t)m * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) st = graph_from_device_edges(ds, dd, n, m, build_flags, graph_flags, out);
  tbfs::dev_free(ds);
  tbfs::dev_free(dd);
  if (e != cudaSuccess) return cuda_fail(e, "edge list upload", __LINE__);
  return st;
}

/* The Matrix Market header of text[0, bytes): banner, comments, size line.
 * *data = offset of the first byte after the size line. */
static tbfs_status mm_header(const char *text, int64_t bytes, long long *M, long long *N,
                             long long *nz, int64_t *data) {
  int64_t p = 0;
  auto line_end = [&](int64_t q) {
    while (q < bytes && text[q] != '\n') ++q;
    return q;
  };
  int64_t e = line_end(0);
  const char banner[] = "%%MatrixMarket";
  if (e < 14 || memcmp(text, banner, 14) != 0) {
    tbfs_set_error("Matrix Market text has no banner");
    return TBFS_ERR_IO;
  }
  bool coord = false;
  for (int64_t q = 0; q + 10 <= e; ++q)
    if (memcmp(text + q, "coordinate", 10) == 0) coord = true;
  if (!coord) {
    tbfs_set_error("Matrix Market text is not a coordinate (sparse) matrix");
    return TBFS_ERR_IO;
  }
  p = e < bytes ? e + 1 : e;
  while (p < bytes) {
    e = line_end(p);
    if (text[p] != '%') {
      char buf[256];
      const int64_t len = e - p < 255 ? e - p : 255;
      memcpy(buf, text + p, (size_t)len);
      buf[len] = 0;
      if (sscanf(buf, "%lld %lld %lld", M, N, nz) == 3) {
        *data = e < bytes ? e + 1 : e;
        if (*M < 0 || *N < 1 || *nz < 0 || *N > INT32_MAX || *M > INT32_MAX) {
          tbfs_set_error("Matrix Market size line out of range");
          return TBFS_ERR_IO;
        }
        return TBFS_OK;
      }
    }
    p = e < bytes ? e + 1 : e;
  }
  tbfs_set_error("Matrix Market text has no size line");
  return TBFS_ERR_IO;
}

extern "C" tbfs_status tbfs_graph_create_mm(const char *text, int64_t bytes, int32_t undirected,
                                            uint32_t build_flags, uint32_t graph_flags,
                                            tbfs_graph **out) {
  if (!out) return invalid("tbfs_graph_create_mm: null out pointer");
  *out = nullptr;
  if (!text || bytes < 1) return invalid("tbfs_graph_create_mm: empty text");
  long long M = 0, N = 0, nz = 0;
  int64_t data = 0;
  tbfs_status st = mm_header(text, bytes, &M, &N, &nz, &data);
  if (st != TBFS_OK) return st;
  if (undirected) build_flags |= TBFS_BUILD_SYMMETRIZE;
  else build_flags &= ~TBFS_BUILD_SYMMETRIZE;
  if (nz > ((build_flags & TBFS_BUILD_SYMMETRIZE) ? INT32_MAX / 2 : INT32_MAX)) {
    tbfs_set_error("tbfs_graph_create_mm: too many entries for int32 lists");
    return TBFS_ERR_UNSUPPORTED;
  }
  if ((st = need_device()) != TBFS_OK) return st;
  const long long len = (long long)(bytes - data);
  char *dt = nullptr;
  int *ds = nullptr, *dd = nullptr;
  const size_t eb = (size_t)(nz > 0 ? nz : 1) * sizeof(int);
  cudaError_t e = tbfs::dev_alloc(&dt, (size_t)(len > 0 ? len : 1));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&ds, eb);
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dd, eb);
  if (e == cudaSuccess && len > 0) e = cudaMemcpy(dt, text + data, (size_t)len, cudaMemcpyHostToDevice);
  long long lines = 0, bad = -1;
  if (e == cudaSuccess) e = tbfs::mm_parse_device(dt, len, nz, M, N, ds, dd, &lines, &bad, 0);
  tbfs::dev_free(dt);
  if (e == cudaSuccess) {
    if (lines < nz) {
      tbfs_set_error("Matrix Market text ends after %lld of %lld entries", lines, nz);
      st = TBFS_ERR_IO;
    } else if (bad >= 0) {
      tbfs_set_error("Matrix Market: bad entry line %lld", bad);
      st = TBFS_ERR_IO;
    } else {
      st = graph_from_device_edges(ds, dd, (int32_t)N, nz, build_flags, graph_flags, out);
    }
  }
  tbfs::dev_free(ds);
  tbfs::dev_free(dd);
  if (e != cudaSuccess) return cuda_fail(e, "Matrix Market parse on the device", __LINE__);
  return st;
}

extern "C" tbfs_status tbfs_graph_load_mm(const char *path, int32_t undirected,
                                          uint32_t build_flags, uint32_t graph_flags,
                                          tbfs_graph **out) {
  if (!out) return invalid("tbfs_graph_load_mm: null out pointer");
  *out = nullptr;
  if (!path) return invalid("tbfs_graph_load_mm: null path");
  FILE *f = fopen(path, "rb");
  if (!f) {
    tbfs_set_error("tbfs_graph_load_mm: cannot open %s", path);
    return TBFS_ERR_IO;
  }
  fseek(f, 0, SEEK_END);
  const long long size = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (size <= 0) {
    fclose(f);
    tbfs_set_error("tbfs_graph_load_mm: %s is empty", path);
    return TBFS_ERR_IO;
  }
  char *text = nullptr; /* pinned: the upload runs at full link speed */
  bool pinned = true;
  if (cudaMallocHost(&text, (size_t)size) != cudaSuccess) {
    cudaGetLastError();
    pinned = false;
    text = static_cast<char *>(malloc((size_t)size));
    if (!text) {
      fclose(f);
      return TBFS_ERR_OUT_OF_MEMORY;
    }
  }
  const size_t got = fread(text, 1, (size_t)size, f);
  fclose(f);
  tbfs_status st = TBFS_ERR_IO;
  if (got != (size_t)size)
    tbfs_set_error("tbfs_graph_load_mm: short read of %s", path);
  else
    st = tbfs_graph_create_mm(text, size, undirected, build_flags, graph_flags, out);
  if (pinned) cudaFreeHost(text);
  else free(text);
  return st;
}

/* The resident in-lists as COOC pairs (row[k] -> col[k], entries in column
 * order, the reference's ICOOC/JCOOC): rows copied, columns expanded on the
 * device.  Same numbering rule as tbfs_graph_get_csc. */
extern "C" tbfs_status tbfs_graph_get_cooc(const tbfs_graph *g, int32_t *row, int32_t *col) {
  if (!g || (g->nnz > 0 && (!row || !col))) return invalid("tbfs_graph_get_cooc: null argument");
  if (g->inv) {
    tbfs_set_error("tbfs_graph_get_cooc: the graph is stored regrouped by degree");
    return TBFS_ERR_UNSUPPORTED;
  }
  if (g->nnz == 0) return TBFS_OK;
  CUDA_TRY(cudaSetDevice(g->device));
  int *dcol = nullptr;
  CUDA_TRY(tbfs::dev_alloc(&dcol, (size_t)g->nnz * sizeof(int)));
  cudaError_t e = tbfs::expand_columns(g->cp, g->n, dcol, 0);
  if (e == cudaSuccess)
    e = cudaMemcpy(col, dcol, (size_t)g->nnz * sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(row, g->ic, (size_t)g->nnz * sizeof(int), cudaMemcpyDeviceToHost);
  tbfs::dev_free(dcol);
  if (e != cudaSuccess) return cuda_fail(e, "tbfs_graph_get_cooc", __LINE__);
  return TBFS_OK;
}

/* The resident in-lists back in the caller's numbering: only for graphs
 * kept in that numbering (TBFS_GRAPH_KEEP_ORDER, or a grouping that left the
 * order unchanged). */
extern "C" tbfs_status tbfs_graph_get_csc(const tbfs_graph *g, int32_t *col_ptr,
                                          int32_t *row_idx) {
  if (!g || !col_ptr || (g->nnz > 0 && !row_idx)) return invalid("tbfs_graph_get_csc: null argument");
  if (g->inv) {
    tbfs_set_error("tbfs_graph_get_csc: the graph is stored regrouped by degree");
    return TBFS_ERR_UNSUPPORTED;
  }
  CUDA_TRY(cudaSetDevice(g->device));
  CUDA_TRY(cudaMemcpy(col_ptr, g->cp, ((size_t)g->n + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  if (g->nnz > 0)
    CUDA_TRY(cudaMemcpy(row_idx, g->ic, (size_t)g->nnz * sizeof(int), cudaMemcpyDeviceToHost));
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_graph_info(const tbfs_graph *g, int32_t *n, int64_t *nnz,
                                       uint32_t *flags) {
  if (!g) return invalid("tbfs_graph_info: null graph");
  if (n) *n = g->n;
  if (nnz) *nnz = g->nnz;
  if (flags) *flags = g->flags;
  return TBFS_OK;
}

/* --------------------------------------------------------- traversal */

static tbfs_status check_opts(const tbfs_graph *g, int32_t root, const tbfs_options &o,
                              const int32_t *S, const int64_t *sigma) {
  if (!g) return invalid("null graph");
  if (root < 0 || root >= g->n) return invalid("root outside [0, n)");
  if (!S) return invalid("null S output");
  if (o.want_sigma && !sigma) return invalid("want_sigma set but sigma output is null");
  if (o.mode < TBFS_MODE_AUTO || o.mode > TBFS_MODE_BOTTOM_UP) return invalid("bad mode");
  if (!(o.alpha > 0.0f) || !(o.beta > 0.0f)) return invalid("alpha and beta must be > 0");
  return TBFS_OK;
}

static tbfs_options resolve_opts(const tbfs_options *in) {
  tbfs_options o;
  tbfs_options_init(&o);
  if (in) o = *in;
  if (o.alpha <= 0.0f) o.alpha = 15.0f;
  if (o.beta <= 0.0f) o.beta = 2.0f;
  if (!(o.pull_ratio > 0.0f)) o.pull_ratio = 1.0f;
  return o;
}

static BfsParams make_params(tbfs_graph *g, int32_t root, const tbfs_options &o, int *S,
                             unsigned long long *sigma) {
  BfsParams p = {};
  p.cp = g->cp;
  p.ic = g->ic;
  p.rp = g->rp;
  p.jr = g->jr;
  p.inv = g->inv;
  p.perm = g->perm;
  p.S_out = S;
  p.sigma_out = o.want_sigma ? sigma : nullptr;
  p.S = g->inv ? g->S_work : S;
  p.sigma = o.want_sigma ? (g->inv ? g->sigma_work : sigma) : nullptr;
  for (int b = 0; b < 3; ++b) {
    p.q[b] = g->queues + (size_t)(0 + b) * g->n;
    p.e[b] = g->queues + (size_t)(3 + b) * g->n;
    p.a[b] = g->queues + (size_t)(6 + b) * g->n;
  }
  for (int b = 0; b < 4; ++b) p.fb[b] = g->bitmaps + (size_t)b * ((g->n + 31) / 32);
  p.ctl = g->ctl;
  p.out_edges_total = g->out_edges_total;
  p.timeout_ns = o.timeout_ns > 0 ? o.timeout_ns : 2000000000LL;
  p.n = g->n;
  p.root = root;
  p.mode = o.mode;
  p.symmetric = g->separate_out ? 0 : 1;
  p.alpha = o.alpha;
  p.beta = o.beta;
  p.pull_ratio = o.pull_ratio;
  p.inject_barrier_skip = o.inject_barrier_skip > 0 ? o.inject_barrier_skip : 0;
  p.trace = nullptr;
  p.trace_cap = 0;
  p.max_ept = o.max_ept;
  p.ctas_per_sm = o.ctas_per_sm;
  p.deg_bits = g->deg_bits;
  p.short_lists = g->short_lists ? 1 : 0;
  return p;
}

/* enqueue: clear control block, time and launch, copy control block back */
static tbfs_status enqueue_bfs(tbfs_graph *g, const BfsParams &p, cudaStream_t s,
                               cudaEvent_t ev0, cudaEvent_t ev1, BfsCtl *ctl_host) {
  CUDA_TRY(cudaMemsetAsync(g->ctl, 0, sizeof(BfsCtl), s));
  CUDA_TRY(cudaEventRecord(ev0, s));
  CUDA_TRY(tbfs::bfs_launch(p, g->geom, s));
  CUDA_TRY(cudaEventRecord(ev1, s));
  CUDA_TRY(cudaMemcpyAsync(ctl_host, g->ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, s));
  return TBFS_OK;
}

/* forward traversal with S / sigma left in the graph's internal numbering
 * (device arrays of n), for consumers inside the library */
tbfs_status tbfs::forward_internal(tbfs_graph *g, int32_t root, const tbfs_options &o, int *S,
                                   unsigned long long *sigma, cudaStream_t s, BfsCtl *ctl_host) {
  BfsParams p = make_params(g, root, o, S, sigma);
  p.S = S;
  p.sigma = o.want_sigma ? sigma : nullptr;
  p.S_out = S;
  p.sigma_out = p.sigma;
  p.perm = nullptr; /* no scatter into the caller's order; inv still maps the root */
  return enqueue_bfs(g, p, s, g->ev0, g->ev1, ctl_host);
}

static tbfs_status stats_from(const BfsCtl &c, cudaEvent_t ev0, cudaEvent_t ev1,
                              tbfs_stats *st) {
  float ms = 0.0f;
  cudaError_t e = cudaEventElapsedTime(&ms, ev0, ev1);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime", __LINE__);
  st->levels = c.levels;
  st->td_levels = c.td_levels;
  st->bu_levels = c.bu_levels;
  st->sigma_overflow = c.sigma_overflow;
  st->visited = c.visited;
  st->edges = c.edges;
  st->device_ms = ms;
  if (c.status != 0) {
    tbfs_set_error("traversal stopped: grid barrier wait exceeded its budget at level %d",
                   c.timeout_level - 2);
    return TBFS_ERR_TIMEOUT;
  }
  return TBFS_OK;
}

static tbfs_status ensure_result_buffers(tbfs_graph *g, bool sigma) {
  if (!g->S_dev) CUDA_TRY(tbfs::dev_alloc(&g->S_dev, (size_t)g->n * sizeof(int)));
  if (sigma && !g->sigma_dev)
    CUDA_TRY(tbfs::dev_alloc(&g->sigma_dev, (size_t)g->n * sizeof(unsigned long long)));
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_graph_last_stats(tbfs_graph *g, tbfs_stats *stats) {
  if (!g || !stats) return invalid("tbfs_graph_last_stats: null argument");
  CUDA_TRY(cudaSetDevice(g->device));
  if (g->pending) {
    CUDA_TRY(cudaStreamSynchronize(g->last_stream));
    g->pending = false;
    tbfs_stats st = {};
    tbfs_status s = stats_from(*g->ctl_host, g->ev0, g->ev1, &st);
    g->last = st;
    g->depth_hint = st.levels;
    if (s != TBFS_OK) {
      *stats = st;
      return s;
    }
  }
  *stats = g->last;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_bfs(tbfs_graph *g, int32_t root, const tbfs_options *opt,
                                int32_t *S, int64_t *sigma, tbfs_stats *stats) {
  const tbfs_options o = resolve_opts(opt);
  tbfs_status st = check_opts(g, root, o, S, sigma);
  if (st != TBFS_OK) return st;
  CUDA_TRY(cudaSetDevice(g->device));
  cudaStream_t s = (cudaStream_t)o.stream;
  int *S_dst = S;
  unsigned long long *sig_dst = reinterpret_cast<unsigned long long *>(sigma);
  if (!o.outputs_on_device) {
    if ((st = ensure_result_buffers(g, o.want_sigma != 0)) != TBFS_OK) return st;
    S_dst = g->S_dev;
    sig_dst = g->sigma_dev;
  }
  BfsParams p = make_params(g, root, o, S_dst, sig_dst);
  const bool tracing = o.level_trace != nullptr && o.level_trace_cap >= 2;
  if (tracing) {
    if (g->trace_cap < o.level_trace_cap) {
      tbfs::dev_free(g->trace_dev);
      g->trace_dev = nullptr;
      g->trace_cap = 0;
      CUDA_TRY(tbfs::dev_alloc(&g->trace_dev, (size_t)o.level_trace_cap * 4 * sizeof(long long)));
      g->trace_cap = o.level_trace_cap;
    }
    CUDA_TRY(cudaMemsetAsync(g->trace_dev, 0, (size_t)o.level_trace_cap * 4 * sizeof(long long), s));
    p.trace = g->trace_dev;
    p.trace_cap = o.level_trace_cap;
  }
  if ((st = enqueue_bfs(g, p, s, g->ev0, g->ev1, g->ctl_host)) != TBFS_OK) return st;
  g->pending = true;
  g->last_stream = s;
  if (tracing)
    CUDA_TRY(cudaMemcpyAsync(o.level_trace, g->trace_dev,
                             (size_t)o.level_trace_cap * 4 * sizeof(long long),
                             cudaMemcpyDeviceToHost, s));
  if (!o.outputs_on_device) {
    CUDA_TRY(cudaMemcpyAsync(S, S_dst, (size_t)g->n * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (o.want_sigma)
      CUDA_TRY(cudaMemcpyAsync(sigma, sig_dst, (size_t)g->n * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, s));
  }
  if (stats || !o.outputs_on_device) {
    tbfs_stats tmp = {};
    st = tbfs_graph_last_stats(g, &tmp);
    if (stats) *stats = tmp;
    return st;
  }
  return TBFS_OK;
}

/* Per-root control blocks and events of tbfs_bfs_many, grown to k roots. */
static tbfs_status many_reserve(tbfs_graph *g, int32_t k) {
  if (g->many_cap >= k) return TBFS_OK;
  tbfs::dev_free(g->many_ctl);
  g->many_ctl = nullptr;
  if (g->many_ctl_host) cudaFreeHost(g->many_ctl_host);
  g->many_ctl_host = nullptr;
  g->many_cap = 0;
  CUDA_TRY(tbfs::dev_alloc(&g->many_ctl, (size_t)k * sizeof(BfsCtl)));
  CUDA_TRY(cudaMallocHost(&g->many_ctl_host, (size_t)k * sizeof(BfsCtl)));
  while (g->many_ev.size() < 2 * (size_t)k) {
    cudaEvent_t x = nullptr;
    CUDA_TRY(cudaEventCreate(&x));
    g->many_ev.push_back(x);
  }
  while (g->many_sync.size() < 2 * (size_t)k) {
    cudaEvent_t x = nullptr;
    CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    g->many_sync.push_back(x);
  }
  g->many_cap = k;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_bfs_many(tbfs_graph *g, const int32_t *roots, int32_t k,
                                     const tbfs_options *opt, int32_t *S, int64_t *sigma,
                                     tbfs_stats *stats) {
  const tbfs_options o = resolve_opts(opt);
  if (!g || !roots || k < 0) return invalid("tbfs_bfs_many: bad arguments");
  if (k == 0) return TBFS_OK;
  for (int32_t i = 0; i < k; ++i) {
    tbfs_status st = check_opts(g, roots[i], o, S, sigma);
    if (st != TBFS_OK) return st;
  }
  CUDA_TRY(cudaSetDevice(g->device));
  cudaStream_t s = (cudaStream_t)o.stream;
  const bool host_out = !o.outputs_on_device;
  const bool want_sigma = o.want_sigma != 0;
  tbfs_status st = TBFS_OK;
  /* host outputs: two device result buffers; the copies of root i run on
   * the copy stream while root i+1 is traversed on s */
  if (host_out) {
    if ((st = ensure_result_buffers(g, want_sigma)) != TBFS_OK) return st;
    if (!g->S_dev2) CUDA_TRY(tbfs::dev_alloc(&g->S_dev2, (size_t)g->n * sizeof(int)));
    if (want_sigma && !g->sigma_dev2)
      CUDA_TRY(tbfs::dev_alloc(&g->sigma_dev2, (size_t)g->n * sizeof(unsigned long long)));
    if (!g->copy_stream) CUDA_TRY(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
  }
  if ((st = many_reserve(g, k)) != TBFS_OK) return st;
  cudaEvent_t *ev = g->many_ev.data();
  cudaEvent_t *ready = g->many_sync.data(), *copied = ready + k;
  BfsCtl *ctl_h = g->many_ctl_host;
  /* the k launches need no stream operation between them but their events:
   * every root has its own control block, all cleared here */
  cudaError_t e = cudaMemsetAsync(g->many_ctl, 0, (size_t)k * sizeof(BfsCtl), s);
  const size_t n = (size_t)g->n;
  for (int32_t i = 0; e == cudaSuccess && st == TBFS_OK && i < k; ++i) {
    int *S_dst;
    unsigned long long *sig_dst;
    if (host_out) {
      S_dst = (i & 1) ? g->S_dev2 : g->S_dev;
      sig_dst = (i & 1) ? g->sigma_dev2 : g->sigma_dev;
      /* the buffer's previous results must be on their way home first */
      if (i >= 2) e = cudaStreamWaitEvent(s, copied[i - 2], 0);
      if (e != cudaSuccess) break;
    } else {
      S_dst = S + i * n;
      sig_dst = reinterpret_cast<unsigned long long *>(sigma) + (want_sigma ? i * n : 0);
    }
    BfsParams p = make_params(g, roots[i], o, S_dst, sig_dst);
    p.ctl = g->many_ctl + i;
    e = cudaEventRecord(ev[2 * i], s);
    if (e == cudaSuccess) e = tbfs::bfs_launch(p, g->geom, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 * i + 1], s);
    if (e == cudaSuccess && host_out) {
      e = cudaEventRecord(ready[i], s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(g->copy_stream, ready[i], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(S + i * n, S_dst, n * sizeof(int), cudaMemcpyDeviceToHost,
                            g->copy_stream);
      if (e == cudaSuccess && want_sigma)
        e = cudaMemcpyAsync(sigma + i * n, sig_dst, n * sizeof(int64_t), cudaMemcpyDeviceToHost,
                            g->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(copied[i], g->copy_stream);
    }
  }
  if (e == cudaSuccess && st == TBFS_OK)
    e = cudaMemcpyAsync(ctl_h, g->many_ctl, (size_t)k * sizeof(BfsCtl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && st == TBFS_OK) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && st == TBFS_OK && host_out) e = cudaStreamSynchronize(g->copy_stream);
  for (int32_t i = 0; e == cudaSuccess && st == TBFS_OK && i < k; ++i) {
    tbfs_stats tmp = {};
    st = stats_from(ctl_h[i], ev[2 * i], ev[2 * i + 1], &tmp);
    if (stats) stats[i] = tmp;
    g->last = tmp;
    g->depth_hint = tmp.levels;
  }
  if (e != cudaSuccess) cudaStreamSynchronize(s); /* nothing of this call left running */
  if (host_out && g->copy_stream) cudaStreamSynchronize(g->copy_stream); /* also on error paths */
  g->pending = false;
  if (e != cudaSuccess) return cuda_fail(e, "tbfs_bfs_many", __LINE__);
  return st;
}

/* ------------------------------------------------------- compat shims */

namespace {

/* What each drop-in entry point hands back (see the table in the header of
 * tbfs_compat.h): the shim converts the engine's exact int32 depths and
 * int64 counts on the device and copies the result straight into the
 * caller's arrays. */
enum CompatKind { K_TD = 0, K_BU = 1, K_TDBU = 2, K_COOC = 3 };

/* TD: S with 0 for unreached (the reference zero-initialises S), float
 * sigma = the exact count rounded once */
__global__ void compat_td_kernel(int *S, const unsigned long long *sg, float *out, int n) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    if (S && S[v] < 0) S[v] = 0;
    out[v] = __ll2float_rn((long long)sg[v]);
  }
}

/* vertices per depth d < cap (shared-memory counters, one global add each) */
__global__ void level_hist_kernel(const int *S, int n, int cap, unsigned long long *cnt) {
  extern __shared__ unsigned h[];
  for (int i = threadIdx.x; i < cap; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = S[v];
    if (d >= 0 && d < cap) atomicAdd(&h[d], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cap; i += blockDim.x)
    if (h[i]) atomicAdd(cnt + i, (unsigned long long)h[i]);
}

/* TDBU: int32 sigma (two's-complement wrap of the count) for the depths the
 * reference expands top-down, 0 beyond */
__global__ void compat_tdbu_kernel(const int *S, const unsigned long long *sg, int *out, int n,
                                   int last_td) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = S[v];
    out[v] = (d >= 0 && d <= last_td) ? (int)(unsigned)sg[v] : 0;
  }
}

int compat_grid(int n) {
  const long long b = ((long long)n + 255) / 256;
  return (int)(b < 2432 ? (b > 0 ? b : 1) : 2432);
}

/* Levels a COOC call runs straight over the pairs before it sorts them
 * into CSC instead (cooc_engine.cu): a level costs one pass over the pairs,
 * the sort a few passes plus the degree grouping. */
constexpr int kCoocMaxLevels = 32;

/* The COOC entry point without the sort: upload the pairs, check them, run
 * `reps` traversals over them, convert sigma to float into sig_h.  *done is
 * false (and nothing is written) when the traversal needs more than
 * kCoocMaxLevels levels. */
tbfs_status cooc_native(const int *I_h, const int *J_h, int r, int nz, int n, int reps,
                        float *sig_h, bool *done) {
  *done = false;
  tbfs_status st0 = need_device();
  if (st0 != TBFS_OK) return st0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  tbfs::LaunchGeom geom;
  if (e == cudaSuccess) e = tbfs::cooc_geometry(dev, &geom);
  if (e != cudaSuccess) return cuda_fail(e, "cooc geometry", __LINE__);
  const size_t nn = (size_t)n, m = nz > 0 ? (size_t)nz : 1, nwords = (nn + 31) / 32;
  int *I = nullptr, *J = nullptr, *S = nullptr, *flag = nullptr;
  unsigned long long *sg = nullptr;
  float *out = nullptr;
  unsigned *fb = nullptr;
  tbfs::CoocCtl *ctl = nullptr;
  e = tbfs::dev_alloc(&I, m * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&J, m * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&S, nn * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&sg, nn * sizeof(unsigned long long));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&out, nn * sizeof(float));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&fb, 3 * nwords * sizeof(unsigned));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&ctl, sizeof(tbfs::CoocCtl));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&flag, sizeof(int));
  if (e == cudaSuccess && nz > 0) e = cudaMemcpy(I, I_h, (size_t)nz * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nz > 0) e = cudaMemcpy(J, J_h, (size_t)nz * sizeof(int), cudaMemcpyHostToDevice);
  int bad = 0;
  if (e == cudaSuccess) e = tbfs::cooc_check(I, J, nz, n, flag, 0);
  if (e == cudaSuccess) e = cudaMemcpy(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost);
  tbfs_status st = TBFS_OK;
  if (e != cudaSuccess) st = cuda_fail(e, "drop-in COOC upload", __LINE__);
  else if (bad) st = invalid("bfs_gpu_td_cooc_sc: a row or column index is outside [0, n)");
  tbfs::CoocParams p = {};
  p.I = I;
  p.J = J;
  p.nnz = nz;
  p.n = n;
  p.root = r;
  p.vec = ((reinterpret_cast<uintptr_t>(I) | reinterpret_cast<uintptr_t>(J)) & 15u) == 0;
  p.max_levels = kCoocMaxLevels;
  p.S = S;
  p.sigma = sg;
  for (int b = 0; b < 3; ++b) p.fb[b] = fb + (size_t)b * nwords;
  p.ctl = ctl;
  p.timeout_ns = 2000000000LL;
  tbfs::CoocCtl c = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double total_ms = 0.0;
  if (st == TBFS_OK) {
    e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
  }
  for (int i = 0; st == TBFS_OK && e == cudaSuccess && i < reps; ++i) {
    e = cudaMemsetAsync(ctl, 0, sizeof(tbfs::CoocCtl), 0);
    if (e == cudaSuccess) e = cudaEventRecord(ev0, 0);
    if (e == cudaSuccess) e = tbfs::cooc_launch(p, geom, 0);
    if (e == cudaSuccess) e = cudaEventRecord(ev1, 0);
    if (e == cudaSuccess) e = cudaMemcpy(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
    total_ms += ms;
    if (e == cudaSuccess && c.status != 0) {
      tbfs_set_error("bfs_gpu_td_cooc_sc: grid barrier wait exceeded its budget at level %d",
                     c.timeout_level - 2);
      st = TBFS_ERR_TIMEOUT;
    }
    if (e == cudaSuccess && c.unfinished) break; /* deeper than the pass budget */
  }
  if (st == TBFS_OK && e == cudaSuccess && !c.unfinished) {
    compat_td_kernel<<<compat_grid(n), 256>>>(nullptr, sg, out, n);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(sig_h, out, nn * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) *done = true;
  }
  if (st == TBFS_OK && e != cudaSuccess) st = cuda_fail(e, "drop-in COOC traversal", __LINE__);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  tbfs::dev_free(flag);
  tbfs::dev_free(ctl);
  tbfs::dev_free(fb);
  tbfs::dev_free(out);
  tbfs::dev_free(sg);
  tbfs::dev_free(S);
  tbfs::dev_free(J);
  tbfs::dev_free(I);
  if (st == TBFS_OK && *done && getenv("TBFS_PRINT_TIMES"))
    printf("tbfs: levels = %d, r = %d, average time BFS = %lfms\n", c.levels, r, total_ms / reps);
  return st;
}

/* Upload (CSC or COOC), run `repetition` traversals on the device (the last
 * one's result is kept, as the reference's drivers keep it), convert and
 * copy into the caller's S_h / sigma_h.  The graph is uploaded as general:
 * the caller's arrays carry no symmetry promise (a symmetric one is
 * recognised on the device and needs no transpose). */
int compat_run(const int *a, const int *b, bool cooc, int r, int nz, int n, int repetition,
               CompatKind kind, int *S_h, void *sig_h) {
  if (n < 1 || nz < 0 || r < 0 || r >= n || (nz > 0 && (!a || !b)) || (!cooc && !b)) {
    tbfs_set_error("invalid arguments: n=%d nz=%d r=%d", n, nz, r);
    return TBFS_ERR_INVALID_ARG;
  }
  const bool want_sigma = kind != K_BU;
  if (kind == K_COOC) { /* shallow graphs: straight over the pairs, no sort */
    bool done = false;
    tbfs_status cs = cooc_native(a, b, r, nz, n, repetition < 1 ? 1 : repetition,
                                 static_cast<float *>(sig_h), &done);
    if (cs != TBFS_OK || done) return cs;
  }
  tbfs_graph *g = nullptr;
  /* the caller's numbering is kept: a graph used for one call does not
   * repay the degree regrouping (RMAT-22: 5.1 vs 6.4 ms per call) */
  tbfs_status st = cooc ? tbfs_graph_create_cooc(a, b, n, nz, TBFS_GRAPH_KEEP_ORDER, &g)
                        : tbfs_graph_create_csc(b, a, n, nz, TBFS_GRAPH_KEEP_ORDER, &g);
  if (st != TBFS_OK) return st;
  int *S = nullptr, *out32 = nullptr;
  unsigned long long *sg = nullptr, *cnt = nullptr;
  cudaError_t e = tbfs::dev_alloc(&S, (size_t)n * sizeof(int));
  if (e == cudaSuccess && want_sigma) e = tbfs::dev_alloc(&sg, (size_t)n * sizeof(unsigned long long));
  if (e == cudaSuccess && want_sigma) e = tbfs::dev_alloc(&out32, (size_t)n * sizeof(int));
  tbfs_options o;
  tbfs_options_init(&o);
  o.want_sigma = want_sigma ? 1 : 0;
  o.outputs_on_device = 1;
  tbfs_stats sts = {};
  double total_ms = 0.0;
  const int reps = repetition < 1 ? 1 : repetition;
  if (e != cudaSuccess) st = cuda_fail(e, "drop-in buffers", __LINE__);
  for (int i = 0; i < reps && st == TBFS_OK; ++i) {
    st = tbfs_bfs(g, r, &o, S, reinterpret_cast<int64_t *>(sg), nullptr);
    if (st == TBFS_OK) st = tbfs_graph_last_stats(g, &sts);
    total_ms += sts.device_ms;
  }
  const int grid = compat_grid(n);
  if (st == TBFS_OK && kind == K_TD) {
    compat_td_kernel<<<grid, 256>>>(S, sg, reinterpret_cast<float *>(out32), n);
    e = cudaGetLastError();
  } else if (st == TBFS_OK && kind == K_COOC) {
    compat_td_kernel<<<grid, 256>>>(nullptr, sg, reinterpret_cast<float *>(out32), n);
    e = cudaGetLastError();
  } else if (st == TBFS_OK && kind == K_TDBU) {
    /* The reference's TDBU drivers keep sigma only for the levels they
     * expand top-down: they stay top-down while the last level held at most
     * 0.001f*n vertices (a float compare, bfsgputdbucsc_sc.cu:112-122) and
     * never switch back, and their bottom-up kernel leaves sigma at 0. */
    const int levels = sts.levels;
    std::vector<unsigned long long> hc((size_t)levels + 1, 0ull);
    const int cap = levels + 1 < 8192 ? levels + 1 : 8192;
    e = tbfs::dev_alloc(&cnt, ((size_t)levels + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(cnt, 0, ((size_t)levels + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) {
      level_hist_kernel<<<grid, 256, (size_t)cap * sizeof(unsigned)>>>(S, n, cap, cnt);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpy(hc.data(), cnt, ((size_t)levels + 1) * sizeof(unsigned long long),
                     cudaMemcpyDeviceToHost);
    const float thr_td = 0.001f;
    const float thresh_td = thr_td * (float)n;
    int last_td = levels; /* deepest level reached top-down */
    for (int d = 1; d < levels && d < cap; ++d)
      if ((float)hc[(size_t)d] > thresh_td) {
        last_td = d;
        break;
      }
    if (levels >= cap && last_td == levels) {
      /* more levels than device counters, none of the first ones past the
       * threshold: count the deeper levels on the host (graphs over 8192
       * levels deep only) */
      std::vector<int> Sh((size_t)n);
      if (e == cudaSuccess) e = cudaMemcpy(Sh.data(), S, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
      std::vector<long long> c2((size_t)levels + 1, 0);
      for (int v = 0; v < n; ++v)
        if (Sh[(size_t)v] >= 0 && Sh[(size_t)v] <= levels) c2[(size_t)Sh[(size_t)v]]++;
      for (int d = cap; d < levels; ++d)
        if ((float)c2[(size_t)d] > thresh_td) {
          last_td = d;
          break;
        }
    }
    if (e == cudaSuccess) {
      compat_tdbu_kernel<<<grid, 256>>>(S, sg, out32, n, last_td);
      e = cudaGetLastError();
    }
  }
  if (st == TBFS_OK && e == cudaSuccess && S_h)
    e = cudaMemcpy(S_h, S, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
  if (st == TBFS_OK && e == cudaSuccess && want_sigma)
    e = cudaMemcpy(sig_h, out32, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
  if (st == TBFS_OK && e != cudaSuccess) st = cuda_fail(e, "drop-in results", __LINE__);
  tbfs::dev_free(cnt);
  tbfs::dev_free(out32);
  tbfs::dev_free(sg);
  tbfs::dev_free(S);
  tbfs_graph_destroy(g);
  if (st == TBFS_OK && getenv("TBFS_PRINT_TIMES"))
    printf("tbfs: levels = %d, r = %d, average time BFS = %lfms\n", sts.levels, r,
           total_ms / reps);
  return st;
}

int td_csc(int *IC_h, int *CP_h, int *S_h, float *sigma_h, int r, int nz, int n, int rep) {
  if (!S_h || !sigma_h) return TBFS_ERR_INVALID_ARG;
  return compat_run(IC_h, CP_h, false, r, nz, n, rep, K_TD, S_h, sigma_h);
}

int bu_csc(int *I_h, int *CP_h, int *S_h, int r, int nz, int n, int rep) {
  if (!S_h) return TBFS_ERR_INVALID_ARG;
  return compat_run(I_h, CP_h, false, r, nz, n, rep, K_BU, S_h, nullptr);
}

int tdbu_csc(int *I_h, int *CP_h, int *S_h, int *sigma_h, int r, int nz, int n, int rep) {
  if (!S_h || !sigma_h) return TBFS_ERR_INVALID_ARG;
  return compat_run(I_h, CP_h, false, r, nz, n, rep, K_TDBU, S_h, sigma_h);
}

}  // namespace

extern "C" int bfs_gpu_td_csc_sc(int *IC_h, int *CP_h, int *S_h, float *sigma_h, int r,
                                 int nz, int n, int repetition) {
  return td_csc(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_td_csc_wa(int *IC_h, int *CP_h, int *S_h, float *sigma_h, int r,
                                 int nz, int n, int repetition) {
  return td_csc(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_bu_csc_sc(int *I_h, int *CP_h, int *S_h, int r, int nz, int n,
                                 int repetition, int bbreak) {
  (void)bbreak;
  return bu_csc(I_h, CP_h, S_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_bu_csc_wa(int *I_h, int *CP_h, int *S_h, int r, int nz, int n,
                                 int repetition, int bbreak) {
  (void)bbreak;
  return bu_csc(I_h, CP_h, S_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_tdbu_csc_sc(int *I_h, int *CP_h, int *S_h, int *sigma_h, int r,
                                   int nz, int n, int repetition, int bbreak) {
  (void)bbreak;
  return tdbu_csc(I_h, CP_h, S_h, sigma_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_tdbu_csc_wa(int *IC_h, int *CP_h, int *S_h, int *sigma_h, int r,
                                   int nz, int n, int repetition, int bbreak) {
  (void)bbreak;
  return tdbu_csc(IC_h, CP_h, S_h, sigma_h, r, nz, n, repetition);
}

extern "C" int bfs_gpu_td_cooc_sc(int *I_h, int *J_h, float *sigma_h, int r, int nz, int n,
                                  int repetition) {
  if (!sigma_h) return TBFS_ERR_INVALID_ARG;
  return compat_run(I_h, J_h, true, r, nz, n, repetition, K_COOC, nullptr, sigma_h);
}
