/*
 * multi_api.cu -- the C ABI over the multi-instance engine (multi_engine.cu):
 *
 *   tbfs_arena_*   many graphs packed in one int32 offset arena, one root
 *                  each, all traversed in one persistent launch;
 *   tbfs_server_*  a request loop on its own host thread: (graph, root)
 *                  queries are admitted into free instance slots while the
 *                  server's device-memory pool has room, advance level by
 *                  level together with the queries already running
 *                  (continuous batching at level granularity), and retire as
 *                  they finish, with their latency recorded.
 *
 * Neither has a counterpart in the reference, which traverses one root of
 * one graph per call (TurboBFS_CSC_TD/bfsgputdcsc_sc.cu:47-149).
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tbfs.h"
#include "tbfs_internal.h"

using tbfs::InstDesc;
using tbfs::LaunchGeom;
using tbfs::MultiCtl;
using tbfs::MultiParams;

namespace {

tbfs_status mfail(cudaError_t e, const char *what) {
  tbfs_set_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
}

#define MTRY(call, what)                             \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return mfail(e_, what);   \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* Per-traversal device buffers inside one block: S, sig, q[3], e[3]. */
size_t inst_bytes(int n, bool sigma) {
  const size_t nn = (size_t)n;
  return align256(nn * 4) + (sigma ? align256(nn * 8) : 0) + 6 * align256(nn * 4);
}

void carve(unsigned char *base, int n, bool sigma, InstDesc &D) {
  const size_t nn = (size_t)n;
  size_t off = 0;
  D.S = reinterpret_cast<int *>(base + off);
  off += align256(nn * 4);
  D.sig = nullptr;
  if (sigma) {
    D.sig = reinterpret_cast<unsigned long long *>(base + off);
    off += align256(nn * 8);
  }
  for (int b = 0; b < 3; ++b) {
    D.q[b] = reinterpret_cast<int *>(base + off);
    off += align256(nn * 4);
    D.e[b] = reinterpret_cast<unsigned *>(base + off);
    off += align256(nn * 4);
  }
}

void fill_stats(const InstDesc &D, float ms, tbfs_stats *st) {
  memset(st, 0, sizeof(*st));
  st->levels = D.levels;
  st->td_levels = D.levels;
  st->bu_levels = 0;
  st->sigma_overflow = D.ovf;
  st->visited = D.visited;
  st->edges = D.edges;
  st->device_ms = ms;
}

/* host-side transpose of one CSC (in-lists) into out-lists */
void transpose_csc(int n, const int32_t *cp, const int32_t *ic, std::vector<int32_t> &rp,
                   std::vector<int32_t> &jr) {
  const int64_t nnz = cp[n];
  rp.assign((size_t)n + 1, 0);
  jr.assign((size_t)nnz, 0);
  for (int64_t k = 0; k < nnz; ++k) rp[(size_t)ic[k] + 1]++;
  for (int v = 0; v < n; ++v) rp[(size_t)v + 1] += rp[(size_t)v];
  std::vector<int32_t> fill(rp.begin(), rp.end() - 1);
  for (int v = 0; v < n; ++v)
    for (int64_t k = cp[v]; k < cp[v + 1]; ++k) jr[(size_t)fill[(size_t)ic[k]]++] = v;
}

}  // namespace

/* =============================================================== arena */

struct tbfs_arena {
  int device = 0;
  int32_t g = 0;
  bool symmetric = false;
  std::vector<int32_t> n;
  std::vector<int64_t> nnz, voff, eoff; /* vertex / entry offsets of graph i */
  std::vector<int> deg_bits;           /* bits of graph i's largest in-degree */
  int64_t nv = 0, ne = 0;
  int *cp = nullptr, *ic = nullptr, *rp = nullptr, *jr = nullptr; /* packed */
  unsigned char *work = nullptr; /* per-graph traversal blocks */
  std::vector<size_t> woff;
  bool work_sigma = false;
  InstDesc *inst = nullptr, *inst_host = nullptr;
  int *slots = nullptr;
  MultiCtl *ctl = nullptr, *ctl_host = nullptr;
  LaunchGeom geom;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void arena_free(tbfs_arena *a) {
  if (!a) return;
  cudaSetDevice(a->device);
  tbfs::dev_free(a->cp);
  tbfs::dev_free(a->ic);
  if (!a->symmetric) {
    tbfs::dev_free(a->rp);
    tbfs::dev_free(a->jr);
  }
  tbfs::dev_free(a->work);
  tbfs::dev_free(a->inst);
  tbfs::dev_free(a->slots);
  tbfs::dev_free(a->ctl);
  if (a->inst_host) cudaFreeHost(a->inst_host);
  if (a->ctl_host) cudaFreeHost(a->ctl_host);
  if (a->ev0) cudaEventDestroy(a->ev0);
  if (a->ev1) cudaEventDestroy(a->ev1);
  delete a;
}

extern "C" void tbfs_arena_destroy(tbfs_arena *a) { arena_free(a); }

static tbfs_status arena_build(tbfs_arena *a, const int32_t *col_ptr, const int32_t *row_idx) {
  MTRY(cudaGetDevice(&a->device), "cudaGetDevice");
  /* validate every graph on the host and pack its out-lists if needed */
  std::vector<int32_t> rp_all, jr_all;
  if (!a->symmetric) {
    rp_all.reserve((size_t)(a->nv + a->g));
    jr_all.reserve((size_t)a->ne);
  }
  for (int32_t i = 0; i < a->g; ++i) {
    const int32_t *cp = col_ptr + a->voff[i] + i;
    const int32_t *ic = row_idx + a->eoff[i];
    const int32_t n = a->n[i];
    if (cp[0] != 0 || cp[n] != a->nnz[i]) {
      tbfs_set_error("tbfs_arena_create: graph %d: col_ptr must start at 0 and end at nnz", i);
      return TBFS_ERR_INVALID_ARG;
    }
    int32_t maxd = 0;
    for (int32_t v = 0; v < n; ++v) {
      if (cp[v + 1] < cp[v]) {
        tbfs_set_error("tbfs_arena_create: graph %d: col_ptr decreases at %d", i, v);
        return TBFS_ERR_INVALID_ARG;
      }
      maxd = std::max(maxd, cp[v + 1] - cp[v]);
    }
    int b = 0;
    while (b < 31 && (1 << b) <= maxd) ++b; /* maxd < 2^b */
    a->deg_bits.push_back(b);
    for (int64_t k = 0; k < a->nnz[i]; ++k)
      if (ic[k] < 0 || ic[k] >= n) {
        tbfs_set_error("tbfs_arena_create: graph %d: row index out of range", i);
        return TBFS_ERR_INVALID_ARG;
      }
    if (!a->symmetric) {
      std::vector<int32_t> rp, jr;
      transpose_csc(n, cp, ic, rp, jr);
      rp_all.insert(rp_all.end(), rp.begin(), rp.end());
      jr_all.insert(jr_all.end(), jr.begin(), jr.end());
    }
  }
  const size_t ncp = (size_t)(a->nv + a->g);
  MTRY(tbfs::dev_alloc(&a->cp, ncp * sizeof(int)), "arena alloc");
  MTRY(tbfs::dev_alloc(&a->ic, std::max<size_t>((size_t)a->ne, 1) * sizeof(int)), "arena alloc");
  MTRY(cudaMemcpy(a->cp, col_ptr, ncp * sizeof(int), cudaMemcpyHostToDevice), "arena upload");
  if (a->ne)
    MTRY(cudaMemcpy(a->ic, row_idx, (size_t)a->ne * sizeof(int), cudaMemcpyHostToDevice),
         "arena upload");
  if (a->symmetric) {
    a->rp = a->cp;
    a->jr = a->ic;
  } else {
    MTRY(tbfs::dev_alloc(&a->rp, ncp * sizeof(int)), "arena alloc");
    MTRY(tbfs::dev_alloc(&a->jr, std::max<size_t>((size_t)a->ne, 1) * sizeof(int)), "arena alloc");
    MTRY(cudaMemcpy(a->rp, rp_all.data(), ncp * sizeof(int), cudaMemcpyHostToDevice),
         "arena upload");
    if (a->ne)
      MTRY(cudaMemcpy(a->jr, jr_all.data(), (size_t)a->ne * sizeof(int), cudaMemcpyHostToDevice),
           "arena upload");
  }
  const int slots = std::min<int32_t>(a->g, tbfs::kMultiMaxSlots);
  MTRY(tbfs::dev_alloc(&a->inst, (size_t)slots * sizeof(InstDesc)), "arena alloc");
  MTRY(cudaMallocHost(&a->inst_host, (size_t)slots * sizeof(InstDesc)), "arena alloc");
  MTRY(tbfs::dev_alloc(&a->slots, (size_t)slots * sizeof(int)), "arena alloc");
  MTRY(tbfs::dev_alloc(&a->ctl, sizeof(MultiCtl)), "arena alloc");
  MTRY(cudaMallocHost(&a->ctl_host, sizeof(MultiCtl)), "arena alloc");
  MTRY(cudaEventCreate(&a->ev0), "event");
  MTRY(cudaEventCreate(&a->ev1), "event");
  MTRY(tbfs::multi_geometry(a->device, &a->geom), "launch geometry");
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_arena_create(int32_t g, const int32_t *n, const int64_t *nnz,
                                         const int32_t *col_ptr, const int32_t *row_idx,
                                         uint32_t flags, tbfs_arena **out) {
  if (!out) return TBFS_ERR_INVALID_ARG;
  *out = nullptr;
  if (g < 1 || !n || !nnz || !col_ptr || !row_idx) {
    tbfs_set_error("tbfs_arena_create: need g >= 1 and all arrays");
    return TBFS_ERR_INVALID_ARG;
  }
  int dc = 0;
  if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) {
    cudaGetLastError();
    tbfs_set_error("no CUDA device visible");
    return TBFS_ERR_NO_DEVICE;
  }
  tbfs_arena *a = new tbfs_arena();
  a->g = g;
  a->symmetric = (flags & TBFS_GRAPH_SYMMETRIC) != 0;
  a->n.assign(n, n + g);
  a->nnz.assign(nnz, nnz + g);
  a->voff.resize((size_t)g);
  a->eoff.resize((size_t)g);
  for (int32_t i = 0; i < g; ++i) {
    if (n[i] < 1 || nnz[i] < 0 || nnz[i] > INT32_MAX) {
      arena_free(a);
      tbfs_set_error("tbfs_arena_create: graph %d: need n >= 1 and 0 <= nnz <= INT32_MAX", i);
      return TBFS_ERR_INVALID_ARG;
    }
    a->voff[(size_t)i] = a->nv;
    a->eoff[(size_t)i] = a->ne;
    a->nv += n[i];
    a->ne += nnz[i];
  }
  if (a->nv + g > INT32_MAX || a->ne > INT32_MAX) {
    arena_free(a);
    tbfs_set_error("tbfs_arena_create: the packed arena exceeds int32 offsets");
    return TBFS_ERR_UNSUPPORTED;
  }
  tbfs_status st = arena_build(a, col_ptr, row_idx);
  if (st != TBFS_OK) {
    arena_free(a);
    return st;
  }
  *out = a;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_arena_info(const tbfs_arena *a, int32_t *g, int64_t *vertices,
                                       int64_t *entries) {
  if (!a) return TBFS_ERR_INVALID_ARG;
  if (g) *g = a->g;
  if (vertices) *vertices = a->nv;
  if (entries) *entries = a->ne;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_arena_bfs(tbfs_arena *a, const int32_t *roots, const tbfs_options *opt,
                                      int32_t *S, int64_t *sigma, tbfs_stats *stats) {
  tbfs_options o;
  tbfs_options_init(&o);
  if (opt) o = *opt;
  if (!a || !roots || !S || (o.want_sigma && !sigma)) {
    tbfs_set_error("tbfs_arena_bfs: null arena, roots or outputs");
    return TBFS_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < a->g; ++i)
    if (roots[i] < 0 || roots[i] >= a->n[(size_t)i]) {
      tbfs_set_error("tbfs_arena_bfs: root of graph %d outside [0, n)", i);
      return TBFS_ERR_INVALID_ARG;
    }
  MTRY(cudaSetDevice(a->device), "cudaSetDevice");
  const bool want_sigma = o.want_sigma != 0;
  cudaStream_t s = (cudaStream_t)o.stream;
  if (!a->work || (want_sigma && !a->work_sigma)) {
    tbfs::dev_free(a->work);
    a->work = nullptr;
    a->woff.assign((size_t)a->g, 0);
    size_t tot = 0;
    for (int32_t i = 0; i < a->g; ++i) {
      a->woff[(size_t)i] = tot;
      tot += inst_bytes(a->n[(size_t)i], want_sigma);
    }
    MTRY(tbfs::dev_alloc(&a->work, tot), "arena traversal buffers");
    a->work_sigma = want_sigma;
  }
  const long long timeout = o.timeout_ns > 0 ? o.timeout_ns : 4000000000LL;
  const int cap = tbfs::kMultiMaxSlots;
  for (int32_t g0 = 0; g0 < a->g; g0 += cap) {
    const int k = std::min<int32_t>(cap, a->g - g0);
    std::vector<int> ids((size_t)k);
    for (int j = 0; j < k; ++j) {
      const int i = g0 + j;
      InstDesc &D = a->inst_host[j];
      memset(&D, 0, sizeof(D));
      D.cp = a->cp + a->voff[(size_t)i] + i;
      D.ic = a->ic + a->eoff[(size_t)i];
      D.rp = a->rp + a->voff[(size_t)i] + i;
      D.jr = a->jr + a->eoff[(size_t)i];
      D.inv = nullptr;
      D.nnz = a->nnz[(size_t)i];
      D.n = a->n[(size_t)i];
      D.deg_bits = a->deg_bits[(size_t)i];
      D.root = roots[i];
      carve(a->work + a->woff[(size_t)i], D.n, want_sigma, D);
      MTRY(cudaMemsetAsync(D.S, 0xff, (size_t)D.n * sizeof(int), s), "clear S");
      if (D.sig) MTRY(cudaMemsetAsync(D.sig, 0, (size_t)D.n * 8, s), "clear sigma");
      ids[(size_t)j] = j;
    }
    MTRY(cudaMemcpyAsync(a->inst, a->inst_host, (size_t)k * sizeof(InstDesc),
                         cudaMemcpyHostToDevice, s),
         "descriptors");
    MTRY(cudaMemcpyAsync(a->slots, ids.data(), (size_t)k * sizeof(int), cudaMemcpyHostToDevice, s),
         "slots");
    MTRY(tbfs::multi_init(a->inst, a->slots, k, s), "init");
    MTRY(cudaMemsetAsync(a->ctl, 0, sizeof(MultiCtl), s), "clear control block");
    MultiParams p;
    p.inst = a->inst;
    p.nslots = k;
    p.max_phases = INT32_MAX;
    p.ctl = a->ctl;
    p.timeout_ns = timeout;
    p.wake = nullptr;
    p.stop_on_done = 0;
    MTRY(cudaEventRecord(a->ev0, s), "event");
    MTRY(tbfs::multi_launch(p, a->geom, s), "multi launch");
    MTRY(cudaEventRecord(a->ev1, s), "event");
    MTRY(cudaMemcpyAsync(a->inst_host, a->inst, (size_t)k * sizeof(InstDesc),
                         cudaMemcpyDeviceToHost, s),
         "read descriptors");
    MTRY(cudaMemcpyAsync(a->ctl_host, a->ctl, sizeof(MultiCtl), cudaMemcpyDeviceToHost, s),
         "read control block");
    /* results: the packed layout is the arena's own (no renumbering) */
    for (int j = 0; j < k; ++j) {
      const int i = g0 + j;
      const InstDesc &D = a->inst_host[j];
      const size_t vo = (size_t)a->voff[(size_t)i];
      const cudaMemcpyKind kind = o.outputs_on_device ? cudaMemcpyDeviceToDevice
                                                      : cudaMemcpyDeviceToHost;
      MTRY(cudaMemcpyAsync(S + vo, D.S, (size_t)D.n * sizeof(int), kind, s), "copy S");
      if (want_sigma)
        MTRY(cudaMemcpyAsync(sigma + vo, D.sig, (size_t)D.n * 8, kind, s), "copy sigma");
    }
    MTRY(cudaStreamSynchronize(s), "arena traversal");
    if (a->ctl_host->status != 0) {
      tbfs_set_error("tbfs_arena_bfs: grid barrier wait exceeded its budget");
      return TBFS_ERR_TIMEOUT;
    }
    float ms = 0.0f;
    MTRY(cudaEventElapsedTime(&ms, a->ev0, a->ev1), "event time");
    if (stats)
      for (int j = 0; j < k; ++j) fill_stats(a->inst_host[j], ms, &stats[g0 + j]);
  }
  return TBFS_OK;
}

/* ============================================================== server */

namespace {

struct Request {
  uint64_t ticket = 0;
  tbfs_graph *g = nullptr;
  int32_t root = 0;
  int32_t *S = nullptr;
  int64_t *sigma = nullptr;
  bool plain = false; /* served by the single-source engine */
  std::chrono::steady_clock::time_point t_submit;
  /* filled on completion */
  bool done = false;
  tbfs_status status = TBFS_OK;
  tbfs_stats stats = {};
  double latency_ms = 0.0;
};

/* first-fit allocator over [0, size) */
class Pool {
 public:
  void reset(size_t size) {
    free_.clear();
    if (size) free_[0] = size;
  }
  bool alloc(size_t bytes, size_t *off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<size_t, size_t> free_;
};

struct Slot {
  bool busy = false;
  std::shared_ptr<Request> req;
  size_t off = 0, bytes = 0;
};

/* A finished multi-instance query whose results were gathered into caller
 * order on the server's stream (event `ready`): the delivery thread copies
 * them to the caller's arrays and then returns the memory block. */
struct Delivery {
  std::shared_ptr<Request> r;
  cudaEvent_t ready = nullptr;
  const int *S_c = nullptr;
  const unsigned long long *sig_c = nullptr;
  int n = 0;
  size_t off = 0, bytes = 0;
  tbfs_stats stats = {};
};

}  // namespace

struct tbfs_server {
  int device = 0;
  int max_slots = 0;
  size_t budget = 0;
  tbfs_options opt;
  unsigned char *mem = nullptr;
  Pool pool;
  std::vector<Slot> slots;
  InstDesc *inst = nullptr, *inst_host = nullptr;
  int *slot_ids = nullptr, *slot_ids_host = nullptr;
  MultiCtl *ctl = nullptr, *ctl_host = nullptr;
  LaunchGeom geom;
  cudaStream_t stream = nullptr;
  /* set by submit, read by the running launch at every level boundary */
  volatile int *wake_host = nullptr;
  int *wake_dev = nullptr;
  /* request queue */
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::deque<std::shared_ptr<Request>> plain_q; /* routed to the single-source engine */
  std::unordered_map<uint64_t, std::shared_ptr<Request>> by_ticket;
  uint64_t next_ticket = 1;
  bool stop = false;
  tbfs_status fatal = TBFS_OK;
  std::thread worker;
  /* result delivery, off the server thread: copies of finished queries run
   * while the next launch does */
  std::deque<Delivery> deliveries;
  std::vector<cudaEvent_t> free_events;
  std::condition_variable cv_deliver;
  /* delivery threads (kDeliverThreads), each with its own copy stream, two
   * pinned staging buffers and their events */
  std::vector<cudaStream_t> copy_streams;
  std::vector<unsigned char *> stage;   /* 2 per thread, kStageBytes each */
  std::vector<cudaEvent_t> stage_ev;    /* 2 per thread */
  std::vector<std::thread> deliverers;
  bool deliver_stop = false;
  bool mem_blocked = false; /* admission waits for memory that deliveries hold */
  /* counters */
  long long launches = 0, levels_run = 0, completed = 0, plain_runs = 0;
  /* host wall time, ns: the server thread in multi-instance launches (enqueue
   * to synchronisation) and in routed single-source queries; the delivery
   * thread copying finished results (overlaps the launches); slot_sum = sum
   * over launches of the slots run */
  long long launch_ns = 0, plain_ns = 0, deliver_ns = 0, slot_sum = 0;
  double device_ms = 0.0;
};

namespace {

/* Where a query runs.  Large graphs whose traversals are shallow (RMAT-like:
 * few levels, huge frontiers) go to the single-source direction-optimizing
 * engine, whose bottom-up levels beat the instances' top-down pushes there;
 * everything else -- small graphs, and deep graphs whose levels are cheap but
 * many -- shares the multi-instance launches.  The depth is that of the
 * graph's last traversal (unknown before the first: then size decides). */
constexpr int kPlainMinVertices = 1 << 17;
/* result-delivery threads per server, and the size of each of their two
 * pinned staging buffers */
constexpr int kDeliverThreads = 2;
constexpr size_t kStageBytes = 16u << 20;
constexpr int kPlainMaxLevels = 48;

bool route_plain(const tbfs_graph *g) {
  return g->n >= kPlainMinVertices && (g->depth_hint == 0 || g->depth_hint <= kPlainMaxLevels);
}

/* Run one routed query on the server's stream.  Its results go to a block of
 * the server's memory and reach the caller through the delivery thread, so
 * the next launch does not wait for the copies; without a free block the
 * query copies straight to the caller's arrays. */
void run_plain(tbfs_server *sv, const std::shared_ptr<Request> &r) {
  tbfs_options o = sv->opt;
  o.want_sigma = r->sigma != nullptr;
  o.stream = sv->stream;
  o.level_trace = nullptr;
  o.level_trace_cap = 0;
  const size_t n = (size_t)r->g->n;
  const size_t need = align256(n * 4) + (r->sigma ? align256(n * 8) : 0);
  size_t off = 0;
  bool staged = false;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    staged = need <= sv->budget && sv->pool.alloc(need, &off);
  }
  const auto t0 = std::chrono::steady_clock::now();
  tbfs_stats st = {};
  tbfs_status rc;
  Delivery dv;
  if (staged) {
    o.outputs_on_device = 1;
    int *S_d = reinterpret_cast<int *>(sv->mem + off);
    int64_t *sig_d = r->sigma ? reinterpret_cast<int64_t *>(sv->mem + off + align256(n * 4)) : nullptr;
    rc = tbfs_bfs(r->g, r->root, &o, S_d, sig_d, &st);
    cudaError_t e = cudaSuccess;
    if (rc == TBFS_OK) {
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (!sv->free_events.empty()) {
          dv.ready = sv->free_events.back();
          sv->free_events.pop_back();
        }
      }
      if (!dv.ready) e = cudaEventCreateWithFlags(&dv.ready, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(dv.ready, sv->stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        rc = TBFS_ERR_CUDA;
      }
    }
    if (rc == TBFS_OK) {
      dv.r = r;
      dv.S_c = S_d;
      dv.sig_c = reinterpret_cast<const unsigned long long *>(sig_d);
      dv.n = (int)n;
      dv.off = off;
      dv.bytes = need;
      dv.stats = st;
    } else {
      cudaStreamSynchronize(sv->stream);
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->pool.release(off, need);
      if (dv.ready) sv->free_events.push_back(dv.ready);
    }
  } else {
    o.outputs_on_device = 0;
    rc = tbfs_bfs(r->g, r->root, &o, r->S, r->sigma, &st);
  }
  const auto now = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->plain_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(now - t0).count();
    sv->plain_runs++;
    if (staged && rc == TBFS_OK) {
      sv->deliveries.push_back(std::move(dv));
    } else {
      r->stats = st;
      r->latency_ms = std::chrono::duration<double, std::milli>(now - r->t_submit).count();
      r->status = rc;
      r->done = true;
      sv->completed++;
    }
  }
  if (staged && rc == TBFS_OK)
    sv->cv_deliver.notify_one();
  else
    sv->cv_done.notify_all();
}

/* one step of the loop: admit, advance every instance up to max_phases
 * levels in one launch, retire the finished ones */
tbfs_status server_step(tbfs_server *sv, bool *idle) {
  std::vector<int> admitted;
  int waiting = 0;
  {
    std::unique_lock<std::mutex> lk(sv->mu);
    sv->mem_blocked = false;
    while (!sv->pending.empty()) {
      auto &r = sv->pending.front();
      if (route_plain(r->g)) {
        r->plain = true;
        sv->plain_q.push_back(r);
        sv->pending.pop_front();
        continue;
      }
      const bool sigma = r->sigma != nullptr;
      const size_t need = inst_bytes(r->g->n, sigma) + align256((size_t)r->g->n * 4) +
                          (sigma ? align256((size_t)r->g->n * 8) : 0); /* + caller-order copy */
      int free_slot = -1;
      for (int i = 0; i < sv->max_slots; ++i)
        if (!sv->slots[(size_t)i].busy) {
          free_slot = i;
          break;
        }
      if (free_slot < 0) break;
      size_t off = 0;
      if (need > sv->budget) { /* can never fit: fail it */
        r->status = TBFS_ERR_OUT_OF_MEMORY;
        r->done = true;
        sv->pending.pop_front();
        sv->cv_done.notify_all();
        continue;
      }
      if (!sv->pool.alloc(need, &off)) { /* wait for memory to be released */
        sv->mem_blocked = true;
        break;
      }
      Slot &sl = sv->slots[(size_t)free_slot];
      sl.busy = true;
      sl.req = r;
      sl.off = off;
      sl.bytes = need;
      admitted.push_back(free_slot);
      sv->pending.pop_front();
    }
    waiting = (int)(sv->pending.size() + sv->plain_q.size());
    *sv->wake_host = 0; /* a submit from now on ends the next launch early */
  }
  cudaStream_t s = sv->stream;
  for (int i : admitted) {
    Slot &sl = sv->slots[(size_t)i];
    const Request &r = *sl.req;
    InstDesc &D = sv->inst_host[i];
    memset(&D, 0, sizeof(D));
    D.cp = r.g->cp;
    D.ic = r.g->ic;
    D.rp = r.g->rp;
    D.jr = r.g->jr;
    D.inv = r.g->inv;
    D.nnz = r.g->nnz;
    D.n = r.g->n;
    D.deg_bits = r.g->deg_bits;
    D.root = r.root;
    carve(sv->mem + sl.off, D.n, r.sigma != nullptr, D);
    MTRY(cudaMemsetAsync(D.S, 0xff, (size_t)D.n * sizeof(int), s), "clear S");
    if (D.sig) MTRY(cudaMemsetAsync(D.sig, 0, (size_t)D.n * 8, s), "clear sigma");
  }
  int nslots = 0;
  for (int i = 0; i < sv->max_slots; ++i) {
    if (sv->slots[(size_t)i].busy)
      nslots = i + 1;
    else
      sv->inst_host[i].done = 1; /* empty */
  }
  *idle = nslots == 0;
  if (nslots == 0) return TBFS_OK;
  MTRY(cudaMemcpyAsync(sv->inst, sv->inst_host, (size_t)nslots * sizeof(InstDesc),
                       cudaMemcpyHostToDevice, s),
       "descriptors");
  if (!admitted.empty()) {
    for (size_t j = 0; j < admitted.size(); ++j) sv->slot_ids_host[j] = admitted[j];
    MTRY(cudaMemcpyAsync(sv->slot_ids, sv->slot_ids_host, admitted.size() * sizeof(int),
                         cudaMemcpyHostToDevice, s),
         "slots");
    MTRY(tbfs::multi_init(sv->inst, sv->slot_ids, (int)admitted.size(), s), "init");
  }
  /* The launch runs until a query finishes (its results are delivered at
   * once and its memory freed) or, unless queries already wait for memory
   * or a slot, until a new query is submitted (it joins at the next level). */
  MultiParams p;
  p.inst = sv->inst;
  p.nslots = nslots;
  p.max_phases = 1 << 20;
  p.ctl = sv->ctl;
  p.timeout_ns = sv->opt.timeout_ns > 0 ? sv->opt.timeout_ns : 4000000000LL;
  p.wake = waiting > 0 ? nullptr : sv->wake_dev;
  p.stop_on_done = 1;
  const auto t_launch = std::chrono::steady_clock::now();
  MTRY(cudaMemsetAsync(sv->ctl, 0, sizeof(MultiCtl), s), "clear control block");
  MTRY(tbfs::multi_launch(p, sv->geom, s), "multi launch");
  MTRY(cudaMemcpyAsync(sv->inst_host, sv->inst, (size_t)nslots * sizeof(InstDesc),
                       cudaMemcpyDeviceToHost, s),
       "read descriptors");
  MTRY(cudaMemcpyAsync(sv->ctl_host, sv->ctl, sizeof(MultiCtl), cudaMemcpyDeviceToHost, s),
       "read control block");
  MTRY(cudaStreamSynchronize(s), "server step");
  const auto t_deliver = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->launches++;
    sv->levels_run += sv->ctl_host->phases;
    sv->slot_sum += nslots;
    sv->launch_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(t_deliver - t_launch).count();
  }
  if (sv->ctl_host->status != 0) {
    tbfs_set_error("tbfs_server: grid barrier wait exceeded its budget");
    return TBFS_ERR_TIMEOUT;
  }
  /* retire: gather each finished query into caller order on this stream and
   * hand it to the delivery thread; its slot is free for the next launch, its
   * memory block once the copies are done */
  std::vector<Delivery> out;
  for (int i = 0; i < nslots; ++i) {
    Slot &sl = sv->slots[(size_t)i];
    if (!sl.busy || !sv->inst_host[i].done) continue;
    const InstDesc &D = sv->inst_host[i];
    /* the caller-order copy sits after the traversal buffers of the block */
    unsigned char *tail = sv->mem + sl.off + inst_bytes(D.n, D.sig != nullptr);
    Delivery dv;
    dv.S_c = reinterpret_cast<const int *>(tail);
    dv.sig_c = D.sig ? reinterpret_cast<const unsigned long long *>(tail + align256((size_t)D.n * 4))
                     : nullptr;
    MTRY(tbfs::multi_gather(D.S, D.sig, D.inv, D.n, const_cast<int *>(dv.S_c),
                            const_cast<unsigned long long *>(dv.sig_c), s),
         "gather");
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      if (!sv->free_events.empty()) {
        dv.ready = sv->free_events.back();
        sv->free_events.pop_back();
      }
    }
    if (!dv.ready) MTRY(cudaEventCreateWithFlags(&dv.ready, cudaEventDisableTiming), "event");
    MTRY(cudaEventRecord(dv.ready, s), "event");
    dv.r = sl.req;
    dv.n = D.n;
    dv.off = sl.off;
    dv.bytes = sl.bytes;
    fill_stats(D, 0.0f, &dv.stats);
    dv.r->g->depth_hint = dv.stats.levels;
    sl.busy = false;
    sl.req.reset();
    out.push_back(std::move(dv));
  }
  if (out.empty()) return TBFS_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (auto &dv : out) sv->deliveries.push_back(std::move(dv));
  }
  if (out.size() > 1)
    sv->cv_deliver.notify_all();
  else
    sv->cv_deliver.notify_one();
  return TBFS_OK;
}

/* Copies finished results to the callers' arrays on the copy stream, in the
 * order they finished, then completes the requests and frees their memory.
 * Returns once stopped and drained. */
/* Device -> caller's (pageable) host memory without a pageable CUDA copy:
 * chunks go by DMA into two pinned staging buffers in turn, and each chunk is
 * copied on by memcpy while the next one is in flight.  The CUDA driver never
 * stages pageable memory here, so this thread's copies do not hold up the
 * server thread's launches. */
cudaError_t copy_to_host(tbfs_server *sv, int idx, cudaStream_t cs, void *dst, const void *src,
                         size_t bytes) {
  unsigned char *buf[2] = {sv->stage[2 * (size_t)idx], sv->stage[2 * (size_t)idx + 1]};
  cudaEvent_t ev[2] = {sv->stage_ev[2 * (size_t)idx], sv->stage_ev[2 * (size_t)idx + 1]};
  const size_t nch = (bytes + kStageBytes - 1) / kStageBytes;
  cudaError_t e = cudaSuccess;
  for (size_t c = 0; c <= nch && e == cudaSuccess; ++c) {
    if (c < nch) { /* chunk c in flight into buffer c % 2 */
      const size_t off = c * kStageBytes, len = std::min(kStageBytes, bytes - off);
      e = cudaMemcpyAsync(buf[c & 1], static_cast<const unsigned char *>(src) + off, len,
                          cudaMemcpyDeviceToHost, cs);
      if (e == cudaSuccess) e = cudaEventRecord(ev[c & 1], cs);
    }
    if (e == cudaSuccess && c > 0) { /* chunk c - 1 on to the caller */
      const size_t p = c - 1, off = p * kStageBytes, len = std::min(kStageBytes, bytes - off);
      e = cudaEventSynchronize(ev[p & 1]);
      if (e == cudaSuccess) memcpy(static_cast<unsigned char *>(dst) + off, buf[p & 1], len);
    }
  }
  return e;
}

void deliver_loop(tbfs_server *sv, int idx) {
  cudaSetDevice(sv->device);
  cudaStream_t cs = sv->copy_streams[(size_t)idx];
  for (;;) {
    Delivery dv;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_deliver.wait(lk, [&] { return sv->deliver_stop || !sv->deliveries.empty(); });
      if (sv->deliveries.empty()) return;
      dv = std::move(sv->deliveries.front());
      sv->deliveries.pop_front();
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaStreamWaitEvent(cs, dv.ready, 0);
    if (e == cudaSuccess) e = copy_to_host(sv, idx, cs, dv.r->S, dv.S_c, (size_t)dv.n * sizeof(int));
    if (e == cudaSuccess && dv.sig_c)
      e = copy_to_host(sv, idx, cs, dv.r->sigma, dv.sig_c, (size_t)dv.n * 8);
    if (e != cudaSuccess) cudaGetLastError();
    const auto now = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      Request &r = *dv.r;
      r.stats = dv.stats;
      r.latency_ms = std::chrono::duration<double, std::milli>(now - r.t_submit).count();
      r.status = e == cudaSuccess ? TBFS_OK : TBFS_ERR_CUDA;
      r.done = true;
      sv->pool.release(dv.off, dv.bytes);
      sv->free_events.push_back(dv.ready);
      sv->completed++;
      sv->deliver_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(now - t0).count();
      sv->mem_blocked = false;
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_one();
  }
}

void server_loop(tbfs_server *sv) {
  cudaSetDevice(sv->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      bool any_busy = false;
      for (const Slot &sl : sv->slots) any_busy |= sl.busy;
      sv->cv_work.wait(lk, [&] {
        return sv->stop || (!sv->pending.empty() && !sv->mem_blocked) || !sv->plain_q.empty() ||
               any_busy;
      });
      if (sv->stop && sv->pending.empty() && sv->plain_q.empty() && !any_busy) return;
      if (sv->stop) {
        /* fail what is still queued, finish nothing new */
        for (auto *q : {&sv->pending, &sv->plain_q})
          for (auto &r : *q) {
            r->status = TBFS_ERR_INVALID_ARG;
            r->done = true;
          }
        sv->pending.clear();
        sv->plain_q.clear();
        sv->cv_done.notify_all();
        if (!any_busy) return;
      }
    }
    bool idle = false;
    tbfs_status st = server_step(sv, &idle);
    /* then one query of the single-source route, if any */
    std::shared_ptr<Request> pr;
    if (st == TBFS_OK) {
      std::lock_guard<std::mutex> lk(sv->mu);
      if (!sv->plain_q.empty()) {
        pr = sv->plain_q.front();
        sv->plain_q.pop_front();
      }
    }
    if (pr) run_plain(sv, pr);
    if (st != TBFS_OK) {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->fatal = st;
      for (Slot &sl : sv->slots)
        if (sl.busy) {
          sl.req->status = st;
          sl.req->done = true;
          sl.busy = false;
          sl.req.reset();
        }
      for (auto *q : {&sv->pending, &sv->plain_q})
        for (auto &r : *q) {
          r->status = st;
          r->done = true;
        }
      sv->pending.clear();
      sv->plain_q.clear();
      sv->cv_done.notify_all();
      return;
    }
  }
}

void server_free(tbfs_server *sv) {
  if (!sv) return;
  cudaSetDevice(sv->device);
  tbfs::dev_free(sv->mem);
  tbfs::dev_free(sv->inst);
  tbfs::dev_free(sv->slot_ids);
  tbfs::dev_free(sv->ctl);
  if (sv->inst_host) cudaFreeHost(sv->inst_host);
  if (sv->slot_ids_host) cudaFreeHost(sv->slot_ids_host);
  if (sv->ctl_host) cudaFreeHost(sv->ctl_host);
  if (sv->wake_host) cudaFreeHost(const_cast<int *>(sv->wake_host));
  if (sv->stream) cudaStreamDestroy(sv->stream);
  for (cudaStream_t x : sv->copy_streams) cudaStreamDestroy(x);
  for (unsigned char *b : sv->stage)
    if (b) cudaFreeHost(b);
  for (cudaEvent_t x : sv->stage_ev)
    if (x) cudaEventDestroy(x);
  for (cudaEvent_t x : sv->free_events) cudaEventDestroy(x);
  delete sv;
}

tbfs_status server_init(tbfs_server *sv) {
  MTRY(cudaGetDevice(&sv->device), "cudaGetDevice");
  MTRY(cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking), "stream");
  for (int i = 0; i < kDeliverThreads; ++i) {
    cudaStream_t x = nullptr;
    MTRY(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), "stream");
    sv->copy_streams.push_back(x);
    for (int b = 0; b < 2; ++b) {
      unsigned char *buf = nullptr;
      MTRY(cudaMallocHost(&buf, kStageBytes), "staging buffer");
      sv->stage.push_back(buf);
      cudaEvent_t ev = nullptr;
      MTRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
      sv->stage_ev.push_back(ev);
    }
  }
  MTRY(tbfs::dev_alloc(&sv->mem, sv->budget), "server memory pool");
  sv->pool.reset(sv->budget);
  MTRY(tbfs::dev_alloc(&sv->inst, (size_t)sv->max_slots * sizeof(InstDesc)), "alloc");
  MTRY(cudaMallocHost(&sv->inst_host, (size_t)sv->max_slots * sizeof(InstDesc)), "alloc");
  memset(sv->inst_host, 0, (size_t)sv->max_slots * sizeof(InstDesc));
  MTRY(tbfs::dev_alloc(&sv->slot_ids, (size_t)sv->max_slots * sizeof(int)), "alloc");
  MTRY(cudaMallocHost(&sv->slot_ids_host, (size_t)sv->max_slots * sizeof(int)), "alloc");
  MTRY(tbfs::dev_alloc(&sv->ctl, sizeof(MultiCtl)), "alloc");
  MTRY(cudaMallocHost(&sv->ctl_host, sizeof(MultiCtl)), "alloc");
  MTRY(tbfs::multi_geometry(sv->device, &sv->geom), "launch geometry");
  int *wh = nullptr;
  MTRY(cudaHostAlloc(&wh, sizeof(int), cudaHostAllocMapped), "wake flag");
  sv->wake_host = wh;
  *sv->wake_host = 0;
  MTRY(cudaHostGetDevicePointer(&sv->wake_dev, wh, 0), "wake flag");
  sv->slots.assign((size_t)sv->max_slots, Slot());
  return TBFS_OK;
}

}  // namespace

extern "C" tbfs_status tbfs_server_create(int32_t max_slots, int64_t mem_budget,
                                          const tbfs_options *opt, tbfs_server **out) {
  if (!out) return TBFS_ERR_INVALID_ARG;
  *out = nullptr;
  if (max_slots < 1 || max_slots > tbfs::kMultiMaxSlots || mem_budget < 1) {
    tbfs_set_error("tbfs_server_create: need 1 <= max_slots <= %d and mem_budget > 0",
                   tbfs::kMultiMaxSlots);
    return TBFS_ERR_INVALID_ARG;
  }
  int dc = 0;
  if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) {
    cudaGetLastError();
    tbfs_set_error("no CUDA device visible");
    return TBFS_ERR_NO_DEVICE;
  }
  tbfs_server *sv = new tbfs_server();
  sv->max_slots = max_slots;
  sv->budget = (size_t)mem_budget;
  tbfs_options_init(&sv->opt);
  if (opt) sv->opt = *opt;
  tbfs_status st = server_init(sv);
  if (st != TBFS_OK) {
    server_free(sv);
    return st;
  }
  for (int i = 0; i < kDeliverThreads; ++i) sv->deliverers.emplace_back(deliver_loop, sv, i);
  sv->worker = std::thread(server_loop, sv);
  *out = sv;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_server_submit(tbfs_server *sv, tbfs_graph *g, int32_t root,
                                          int32_t *S, int64_t *sigma, uint64_t *ticket) {
  if (!sv || !g || !S || !ticket) {
    tbfs_set_error("tbfs_server_submit: null server, graph, S or ticket");
    return TBFS_ERR_INVALID_ARG;
  }
  if (root < 0 || root >= g->n) {
    tbfs_set_error("tbfs_server_submit: root outside [0, n)");
    return TBFS_ERR_INVALID_ARG;
  }
  if (g->device != sv->device) {
    tbfs_set_error("tbfs_server_submit: graph lives on another device");
    return TBFS_ERR_INVALID_ARG;
  }
  auto r = std::make_shared<Request>();
  r->g = g;
  r->root = root;
  r->S = S;
  r->sigma = sigma;
  r->t_submit = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop || sv->fatal != TBFS_OK) {
      tbfs_set_error("tbfs_server_submit: server stopped");
      return sv->fatal != TBFS_OK ? sv->fatal : TBFS_ERR_INVALID_ARG;
    }
    r->ticket = sv->next_ticket++;
    sv->by_ticket[r->ticket] = r;
    sv->pending.push_back(r);
    *sv->wake_host = 1;
  }
  sv->cv_work.notify_one();
  *ticket = r->ticket;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_server_wait(tbfs_server *sv, uint64_t ticket, tbfs_stats *stats,
                                        double *latency_ms) {
  if (!sv) return TBFS_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->by_ticket.find(ticket);
  if (it == sv->by_ticket.end()) {
    tbfs_set_error("tbfs_server_wait: unknown ticket");
    return TBFS_ERR_INVALID_ARG;
  }
  std::shared_ptr<Request> r = it->second;
  sv->cv_done.wait(lk, [&] { return r->done; });
  sv->by_ticket.erase(it);
  if (stats) *stats = r->stats;
  if (latency_ms) *latency_ms = r->latency_ms;
  return r->status;
}

extern "C" tbfs_status tbfs_server_counters(tbfs_server *sv, int64_t *launches, int64_t *levels,
                                            int64_t *completed) {
  if (!sv) return TBFS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (launches) *launches = sv->launches;
  if (levels) *levels = sv->levels_run;
  if (completed) *completed = sv->completed;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_server_time_split(tbfs_server *sv, double *launch_ms, double *plain_ms,
                                              double *deliver_ms, int64_t *plain_runs,
                                              int64_t *slot_sum) {
  if (!sv) return TBFS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (launch_ms) *launch_ms = 1e-6 * (double)sv->launch_ns;
  if (plain_ms) *plain_ms = 1e-6 * (double)sv->plain_ns;
  if (deliver_ms) *deliver_ms = 1e-6 * (double)sv->deliver_ns;
  if (plain_runs) *plain_runs = sv->plain_runs;
  if (slot_sum) *slot_sum = sv->slot_sum;
  return TBFS_OK;
}

extern "C" void tbfs_server_destroy(tbfs_server *sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable()) sv->worker.join();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->deliver_stop = true;
  }
  sv->cv_deliver.notify_all();
  for (std::thread &t : sv->deliverers)
    if (t.joinable()) t.join();
  server_free(sv);
}
