/*
 * tune.cu -- degree profile of a resident graph (on the device) and the
 * autotuner of the traversal parameters keyed by it.
 *
 * Degree profile: hist[b] = vertices whose in-degree d has floor(log2(d+1))
 * == b (b < 40), the maximum and the mean, by one pass over col_ptr with
 * block-aggregated histograms: the key of the autotuner's cache.
 *
 * Degree statistics (tbfs_graph_degree_stats): what the reference's drivers
 * print from TurboBFS_CSC_TD/degree.c:22-141 -- the degree vector
 * (degree_ug: out + in of the file entries; in- or out-degree alone),
 * its maximum and the first vertex holding it (degree_max), mean and sample
 * standard deviation (degree_sta), and the per-degree and accumulated log2
 * distributions with their percentages (degree_dist, degree_dist_rel,
 * degree_dist_ac).  The device makes two passes over the lists' pointers:
 * maximum and sum, then the per-degree histogram (shared-memory counters for
 * small degrees) and the first vertex of maximum degree in the caller's
 * numbering.  The host finishes from the histogram in degree order, so the
 * accumulated distributions are the reference's to the bit.
 *
 * Autotuner: the single-source engine's shape (list entries per lane and
 * round, CTAs per SM), then its direction switch (alpha, beta) and path-count
 * schedule (pull_ratio) are chosen by timing traversals from sample roots
 * (CUDA events) over a small grid of candidates; the frontier-matrix batch's
 * push/pull threshold likewise by timing batch launches.  The winner is
 * cached under a key made of the profile's shape (log2 of n, nnz and the
 * maximum degree, and every histogram bucket rounded to a power of two; for
 * the batch also the root count rounded up to a power of two): graphs of one
 * family and scale share it, so a later call returns without timing.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "tbfs.h"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

constexpr int kBuckets = 40;

__global__ void degree_profile_kernel(const int *cp, int n, unsigned long long *hist,
                                      int *maxdeg) {
  __shared__ unsigned h[kBuckets];
  __shared__ int mx;
  if (threadIdx.x < kBuckets) h[threadIdx.x] = 0;
  if (threadIdx.x == 0) mx = 0;
  __syncthreads();
  int lmax = 0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = cp[v + 1] - cp[v];
    const int b = 31 - __clz((unsigned)d + 1u); /* floor(log2(d + 1)) */
    atomicAdd(&h[b], 1u);
    lmax = max(lmax, d);
  }
  atomicMax(&mx, lmax);
  __syncthreads();
  if (threadIdx.x < kBuckets && h[threadIdx.x]) atomicAdd(hist + threadIdx.x, (unsigned long long)h[threadIdx.x]);
  if (threadIdx.x == 0) atomicMax(maxdeg, mx);
}

/* degree of internal vertex v: in (cp), out (rp), or the undirected degree
 * (in-list length of a symmetric graph, in + out otherwise) */
__device__ __forceinline__ int vertex_degree(const int *cp, const int *rp, int kind, bool sym,
                                             int v) {
  const int din = __ldg(cp + v + 1) - __ldg(cp + v);
  if (kind == TBFS_DEGREE_IN || (kind == TBFS_DEGREE_UNDIRECTED && sym)) return din;
  const int dout = __ldg(rp + v + 1) - __ldg(rp + v);
  return kind == TBFS_DEGREE_OUT ? dout : din + dout;
}

/* pass 1: maximum and sum of the degrees */
__global__ void degree_max_sum_kernel(const int *cp, const int *rp, int kind, bool sym, int n,
                                      unsigned long long *sum, int *maxdeg) {
  __shared__ unsigned long long s_sum;
  __shared__ int s_max;
  if (threadIdx.x == 0) {
    s_sum = 0;
    s_max = 0;
  }
  __syncthreads();
  unsigned long long ls = 0;
  int lm = 0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = vertex_degree(cp, rp, kind, sym, (int)v);
    ls += (unsigned long long)d;
    lm = max(lm, d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ls += __shfl_xor_sync(0xffffffffu, ls, o);
    lm = max(lm, __shfl_xor_sync(0xffffffffu, lm, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_sum, ls);
    atomicMax(&s_max, lm);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(sum, s_sum);
    atomicMax(maxdeg, s_max);
  }
}

/* pass 2: hist[d] = vertices of degree d (d <= maxd), counted in shared
 * memory below kSmallDeg; *argmax = smallest caller id of maximum degree */
constexpr int kSmallDeg = 2048;
__global__ void degree_hist_kernel(const int *cp, const int *rp, int kind, bool sym, int n,
                                   const int *perm, int maxd, unsigned long long *hist,
                                   int *argmax) {
  __shared__ unsigned h[kSmallDeg];
  for (int i = threadIdx.x; i < kSmallDeg; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = vertex_degree(cp, rp, kind, sym, (int)v);
    if (d < kSmallDeg) atomicAdd(&h[d], 1u);
    else atomicAdd(hist + d, 1ull);
    if (d == maxd) atomicMin(argmax, perm ? __ldg(perm + v) : (int)v);
  }
  __syncthreads();
  const int lim = maxd + 1 < kSmallDeg ? maxd + 1 : kSmallDeg;
  for (int i = threadIdx.x; i < lim; i += blockDim.x)
    if (h[i]) atomicAdd(hist + i, (unsigned long long)h[i]);
}

std::mutex g_cache_mu;

std::string profile_key(const tbfs_graph *g, const int64_t *hist, int64_t maxd) {
  auto lg = [](double x) { return x < 1 ? 0 : (int)std::floor(std::log2(x)); };
  char buf[512];
  int o = snprintf(buf, sizeof buf, "n%d_m%d_x%d_", lg((double)g->n), lg((double)g->nnz),
                   lg((double)maxd));
  for (int b = 0; b < kBuckets && o < (int)sizeof(buf) - 4; ++b)
    o += snprintf(buf + o, sizeof(buf) - (size_t)o, "%x", (unsigned)lg((double)hist[b] + 1.0) & 31u);
  return std::string(buf) + (g->separate_out ? "_dir" : "_sym");
}

/* a cache line: "key alpha beta pull_ratio [max_ept ctas_per_sm]" */
struct Tuned {
  float a = 15.0f, b = 2.0f, pr = 1.0f;
  int ept = 0, ctas = 0;
};

bool cache_lookup(const char *path, const std::string &key, Tuned *t) {
  if (!path) return false;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  FILE *f = fopen(path, "r");
  if (!f) return false;
  char line[1024], k[512];
  bool found = false;
  while (fgets(line, sizeof line, f)) {
    Tuned x;
    const int got = sscanf(line, "%511s %f %f %f %d %d", k, &x.a, &x.b, &x.pr, &x.ept, &x.ctas);
    if (got >= 4 && key == k) { /* the last entry for the key wins */
      if (got < 6) x.ept = x.ctas = 0;
      *t = x;
      found = true;
    }
  }
  fclose(f);
  return found;
}

void cache_store(const char *path, const std::string &key, const Tuned &t) {
  if (!path) return;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %g %g %g %d %d\n", key.c_str(), t.a, t.b, t.pr, t.ept, t.ctas);
  fclose(f);
}

}  // namespace

cudaError_t longest_list(const int *ptr, int n, int *out) {
  unsigned long long *dh = nullptr;
  cudaError_t e = dev_alloc(&dh, kBuckets * sizeof(unsigned long long) + sizeof(int));
  int *dm = reinterpret_cast<int *>(dh + kBuckets);
  if (e == cudaSuccess) e = cudaMemset(dh, 0, kBuckets * sizeof(unsigned long long) + sizeof(int));
  if (e == cudaSuccess) {
    const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, 4096);
    degree_profile_kernel<<<blocks, 256>>>(ptr, n, dh, dm);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dm, sizeof(int), cudaMemcpyDeviceToHost);
  if (dh) dev_free(dh);
  return e;
}

}  // namespace tbfs

extern "C" tbfs_status tbfs_graph_degree_profile(tbfs_graph *g, int64_t *hist40,
                                                 int64_t *max_degree, double *mean_degree) {
  if (!g || !hist40) {
    tbfs_set_error("tbfs_graph_degree_profile: null graph or histogram");
    return TBFS_ERR_INVALID_ARG;
  }
  cudaError_t e = cudaSetDevice(g->device);
  unsigned long long *dh = nullptr;
  int *dm = nullptr;
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dh, tbfs::kBuckets * sizeof(unsigned long long) + sizeof(int));
  if (e == cudaSuccess) {
    dm = reinterpret_cast<int *>(dh + tbfs::kBuckets);
    e = cudaMemset(dh, 0, tbfs::kBuckets * sizeof(unsigned long long) + sizeof(int));
  }
  if (e == cudaSuccess) {
    const int blocks = (int)std::min<long long>(((long long)g->n + 255) / 256, 4096);
    tbfs::degree_profile_kernel<<<blocks, 256>>>(g->cp, g->n, dh, dm);
    e = cudaGetLastError();
  }
  unsigned long long h[tbfs::kBuckets];
  int mx = 0;
  if (e == cudaSuccess) e = cudaMemcpy(h, dh, sizeof h, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&mx, dm, sizeof mx, cudaMemcpyDeviceToHost);
  tbfs::dev_free(dh);
  if (e != cudaSuccess) {
    tbfs_set_error("tbfs_graph_degree_profile: %s", cudaGetErrorString(e));
    return TBFS_ERR_CUDA;
  }
  for (int b = 0; b < tbfs::kBuckets; ++b) hist40[b] = (int64_t)h[b];
  if (max_degree) *max_degree = mx;
  if (mean_degree) *mean_degree = g->n ? (double)g->nnz / (double)g->n : 0.0;
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_graph_degree_stats(tbfs_graph *g, int32_t kind,
                                               tbfs_degree_stats *out, int64_t *dist,
                                               int64_t dist_cap) {
  if (!g || !out || kind < TBFS_DEGREE_IN || kind > TBFS_DEGREE_UNDIRECTED ||
      (dist && dist_cap < 0)) {
    tbfs_set_error("tbfs_graph_degree_stats: null graph or output, or unknown degree kind");
    return TBFS_ERR_INVALID_ARG;
  }
  memset(out, 0, sizeof *out);
  out->argmax = -1;
  const int n = g->n;
  if (n == 0) return TBFS_OK;
  /* degree_ug's out + in counts each entry of a declared-undirected graph
   * once (the file holds one triangle), of any other graph at both ends */
  const bool sym = g->declared_symmetric;
  const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, 1216);
  cudaError_t e = cudaSetDevice(g->device);
  unsigned long long *dsum = nullptr, *hist = nullptr;
  int *dmax = nullptr;
  unsigned long long hsum = 0;
  int hmax = 0, harg = -1;
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dsum, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    dmax = reinterpret_cast<int *>(dsum + 1);
    e = cudaMemset(dsum, 0, 2 * sizeof(unsigned long long));
  }
  if (e == cudaSuccess) {
    tbfs::degree_max_sum_kernel<<<blocks, 256>>>(g->cp, g->rp, kind, sym, n, dsum, dmax);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&hsum, dsum, sizeof hsum, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&hmax, dmax, sizeof hmax, cudaMemcpyDeviceToHost);
  /* histogram of hmax + 1 counters, then the argmax word */
  const size_t hbytes = ((size_t)hmax + 1) * sizeof(unsigned long long);
  if (e == cudaSuccess) e = tbfs::dev_alloc(&hist, hbytes + sizeof(unsigned long long));
  int *darg = hist ? reinterpret_cast<int *>(reinterpret_cast<char *>(hist) + hbytes) : nullptr;
  if (e == cudaSuccess) e = cudaMemset(hist, 0, hbytes);
  if (e == cudaSuccess) e = cudaMemset(darg, 0x7f, sizeof(int));
  if (e == cudaSuccess) {
    tbfs::degree_hist_kernel<<<blocks, 256>>>(g->cp, g->rp, kind, sym, n, g->perm, hmax, hist,
                                               darg);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> h((size_t)hmax + 1);
  if (e == cudaSuccess) e = cudaMemcpy(h.data(), hist, hbytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&harg, darg, sizeof harg, cudaMemcpyDeviceToHost);
  tbfs::dev_free(hist);
  tbfs::dev_free(dsum);
  if (e != cudaSuccess) {
    tbfs_set_error("tbfs_graph_degree_stats: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
  }
  /* host side, in degree order as degree.c:54-141 */
  out->max_degree = hmax;
  out->argmax = hmax > 0 ? harg : -1;
  out->sum = (int64_t)hsum;
  out->mean = (double)hsum / (double)n;
  double ss = 0.0;
  for (int d = 0; d <= hmax; ++d)
    if (h[(size_t)d]) ss += (double)h[(size_t)d] * std::pow((double)d - out->mean, 2);
  out->sd = std::sqrt(ss / (double)(n - 1));
  std::vector<double> rel((size_t)hmax + 1);
  for (int d = 0; d <= hmax; ++d) rel[(size_t)d] = (double)h[(size_t)d] * 100.0 / ((double)n);
  for (int b = 0; b < 2 && b <= hmax; ++b) {
    out->dist_ac[b] = (int64_t)h[(size_t)b];
    out->dist_rel_ac[b] = rel[(size_t)b];
  }
  int b = 2;
  for (long long low = 2; low < hmax && b < TBFS_DEGREE_BUCKETS; low *= 2, ++b)
    for (long long d = low; d < 2 * low && d <= hmax; ++d) {
      out->dist_ac[b] += (int64_t)h[(size_t)d];
      out->dist_rel_ac[b] += rel[(size_t)d];
    }
  if (dist)
    for (int64_t d = 0; d < dist_cap && d <= hmax; ++d) dist[d] = (int64_t)h[(size_t)d];
  return TBFS_OK;
}

static void apply(const tbfs::Tuned &t, tbfs_options *o) {
  o->alpha = t.a;
  o->beta = t.b;
  o->pull_ratio = t.pr;
  o->max_ept = t.ept;
  o->ctas_per_sm = t.ctas;
}

extern "C" tbfs_status tbfs_autotune(tbfs_graph *g, const int32_t *roots, int32_t k,
                                     const char *cache_path, tbfs_options *opt,
                                     int32_t *from_cache) {
  if (!g || !opt || k < 1 || !roots) {
    tbfs_set_error("tbfs_autotune: need a graph, options and at least one root");
    return TBFS_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) {
      tbfs_set_error("tbfs_autotune: root outside [0, n)");
      return TBFS_ERR_INVALID_ARG;
    }
  int64_t hist[tbfs::kBuckets], maxd = 0;
  tbfs_status st = tbfs_graph_degree_profile(g, hist, &maxd, nullptr);
  if (st != TBFS_OK) return st;
  const std::string key = tbfs::profile_key(g, hist, maxd);
  tbfs::Tuned best;
  if (from_cache) *from_cache = 0;
  if (tbfs::cache_lookup(cache_path, key, &best)) {
    apply(best, opt);
    if (from_cache) *from_cache = 1;
    return TBFS_OK;
  }
  /* time one setting: device time of k traversals, outputs on the device */
  int *S = nullptr;
  unsigned long long *sg = nullptr;
  if (tbfs::dev_alloc(&S, (size_t)k * g->n * sizeof(int)) != cudaSuccess ||
      tbfs::dev_alloc(&sg, (size_t)k * g->n * sizeof(unsigned long long)) != cudaSuccess) {
    tbfs::dev_free(S);
    tbfs_set_error("tbfs_autotune: out of device memory for the sample outputs");
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  std::vector<tbfs_stats> sts((size_t)k);
  tbfs_options base = *opt;
  base.outputs_on_device = 1;
  base.level_trace = nullptr;
  base.level_trace_cap = 0;
  auto time_of = [&](const tbfs::Tuned &t, double *ms) -> tbfs_status {
    tbfs_options o = base;
    apply(t, &o);
    double b = 1e30;
    for (int rep = 0; rep < 2; ++rep) { /* the better of two runs */
      tbfs_status s2 = tbfs_bfs_many(g, roots, k, &o, S, reinterpret_cast<int64_t *>(sg), sts.data());
      if (s2 != TBFS_OK) return s2;
      double t2 = 0.0;
      for (const auto &x : sts) t2 += x.device_ms;
      b = std::min(b, t2);
    }
    *ms = b;
    return TBFS_OK;
  };
  double cur = 0.0;
  st = time_of(best, &cur);
  auto consider = [&](const tbfs::Tuned &t) {
    double ms = 0.0;
    if (st != TBFS_OK) return;
    if ((st = time_of(t, &ms)) == TBFS_OK && ms < cur) {
      cur = ms;
      best = t;
    }
  };
  /* stage 1, the engine's shape at the default direction parameters: list
   * entries per lane and round, CTAs per SM */
  const int epts[] = {2, 4, 0};
  const int ctass[] = {1, 2, 4}; /* 4 = every CTA that fits (0 means 2 on short-list graphs) */
  const tbfs::Tuned s0 = best;
  for (int e : epts)
    for (int c : ctass) {
      tbfs::Tuned t = s0;
      t.ept = e;
      t.ctas = c;
      if (t.ept != s0.ept || t.ctas != s0.ctas) consider(t);
    }
  /* stage 2, every combination of a grid of the direction switch and the
   * path-count schedule at that shape (a coordinate search over wider lists
   * stalled in a local optimum on RMAT) */
  const float alphas[] = {4.0f, 6.0f, 9.0f, 12.0f, 15.0f, 24.0f, 60.0f};
  const float betas[] = {1.0f, 2.0f, 4.0f, 18.0f};
  const float ratios[] = {0.5f, 1.0f, 2.0f, 4.0f};
  const tbfs::Tuned s1 = best;
  for (float xa : alphas)
    for (float xb : betas)
      for (float xp : ratios) {
        tbfs::Tuned t = s1;
        t.a = xa;
        t.b = xb;
        t.pr = xp;
        if (xa != s1.a || xb != s1.b || xp != s1.pr) consider(t);
      }
  tbfs::dev_free(S);
  tbfs::dev_free(sg);
  if (st != TBFS_OK) return st;
  apply(best, opt);
  tbfs::cache_store(cache_path, key, best);
  return TBFS_OK;
}

extern "C" tbfs_status tbfs_autotune_batch(tbfs_graph *g, const int32_t *roots, int32_t k,
                                           const char *cache_path, tbfs_options *opt,
                                           int32_t *from_cache) {
  if (!g || !opt || k < 1 || k > TBFS_BATCH_MAX_ROOTS || !roots) {
    tbfs_set_error("tbfs_autotune_batch: need a graph, options and 1..256 roots");
    return TBFS_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) {
      tbfs_set_error("tbfs_autotune_batch: root outside [0, n)");
      return TBFS_ERR_INVALID_ARG;
    }
  int64_t hist[tbfs::kBuckets], maxd = 0;
  tbfs_status st = tbfs_graph_degree_profile(g, hist, &maxd, nullptr);
  if (st != TBFS_OK) return st;
  int kb = 1;
  while (kb < k) kb *= 2;
  const std::string key = tbfs::profile_key(g, hist, maxd) + "_batch" + std::to_string(kb) +
                          (opt->want_sigma ? "s" : "d");
  tbfs::Tuned t;
  if (from_cache) *from_cache = 0;
  if (tbfs::cache_lookup(cache_path, key, &t)) {
    opt->alpha = t.a;
    if (from_cache) *from_cache = 1;
    return TBFS_OK;
  }
  int *S = nullptr;
  unsigned long long *sg = nullptr;
  if (tbfs::dev_alloc(&S, (size_t)k * g->n * sizeof(int)) != cudaSuccess ||
      (opt->want_sigma &&
       tbfs::dev_alloc(&sg, (size_t)k * g->n * sizeof(unsigned long long)) != cudaSuccess)) {
    tbfs::dev_free(S);
    tbfs_set_error("tbfs_autotune_batch: out of device memory for the sample outputs");
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  std::vector<tbfs_stats> sts((size_t)k);
  tbfs_options o = *opt;
  o.outputs_on_device = 1;
  o.level_trace = nullptr;
  o.level_trace_cap = 0;
  /* the push/pull threshold of the frontier-matrix batch; one launch per
   * setting, the better of two */
  const float alphas[] = {3.0f, 5.0f, 8.0f, 15.0f, 30.0f};
  double best_ms = 1e30;
  float best_a = opt->alpha > 0.0f ? opt->alpha : 15.0f;
  for (float a : alphas) {
    o.alpha = a;
    double ms = 1e30;
    for (int rep = 0; rep < 2 && st == TBFS_OK; ++rep) {
      st = tbfs_bfs_batch(g, roots, k, &o, TBFS_LAYOUT_ROOT_MAJOR, S,
                          reinterpret_cast<int64_t *>(sg), sts.data());
      if (st == TBFS_OK) ms = std::min(ms, sts[0].device_ms);
    }
    if (st != TBFS_OK) break;
    if (ms < best_ms) {
      best_ms = ms;
      best_a = a;
    }
  }
  tbfs::dev_free(S);
  tbfs::dev_free(sg);
  if (st != TBFS_OK) return st;
  opt->alpha = best_a;
  t.a = best_a;
  tbfs::cache_store(cache_path, key, t);
  return TBFS_OK;
}
