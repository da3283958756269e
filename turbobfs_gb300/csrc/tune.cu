/*
 * tune.cu -- degree profile of a resident graph (on the device) and the
 * autotuner of the traversal parameters keyed by it.
 *
 * Degree profile: hist[b] = vertices whose in-degree d has floor(log2(d+1))
 * == b (b < 40), the maximum and the mean -- the statistics the reference
 * prints from its host code (TurboBFS_CSC_TD/degree.c:22-141), computed
 * here by one pass over col_ptr with block-aggregated histograms.
 *
 * Autotuner: the direction switch (alpha, beta) and the path-count schedule
 * (pull_ratio) of the single-source engine are chosen by timing traversals
 * from sample roots (CUDA events) for every combination of a small grid of
 * candidates (and the defaults).  The winner is cached under a
 * key made of the profile's shape (log2 of n, nnz and the maximum degree,
 * and every histogram bucket rounded to a power of two): graphs of one
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

bool cache_lookup(const char *path, const std::string &key, float *a, float *b, float *pr) {
  if (!path) return false;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  FILE *f = fopen(path, "r");
  if (!f) return false;
  char k[512];
  float x, y, z;
  bool found = false;
  while (fscanf(f, "%511s %f %f %f", k, &x, &y, &z) == 4)
    if (key == k) { /* the last entry for the key wins */
      *a = x;
      *b = y;
      *pr = z;
      found = true;
    }
  fclose(f);
  return found;
}

void cache_store(const char *path, const std::string &key, float a, float b, float pr) {
  if (!path) return;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %g %g %g\n", key.c_str(), a, b, pr);
  fclose(f);
}

}  // namespace
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
  float a = 15.0f, b = 18.0f, pr = 4.0f;
  if (from_cache) *from_cache = 0;
  if (tbfs::cache_lookup(cache_path, key, &a, &b, &pr)) {
    opt->alpha = a;
    opt->beta = b;
    opt->pull_ratio = pr;
    if (from_cache) *from_cache = 1;
    return TBFS_OK;
  }
  /* time one parameter set: device time of k traversals, outputs on the device */
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
  auto time_of = [&](float ta, float tb, float tp, double *ms) -> tbfs_status {
    tbfs_options o = base;
    o.alpha = ta;
    o.beta = tb;
    o.pull_ratio = tp;
    double best = 1e30;
    for (int rep = 0; rep < 2; ++rep) { /* the better of two runs */
      tbfs_status s2 = tbfs_bfs_many(g, roots, k, &o, S, reinterpret_cast<int64_t *>(sg), sts.data());
      if (s2 != TBFS_OK) return s2;
      double t = 0.0;
      for (const auto &x : sts) t += x.device_ms;
      best = std::min(best, t);
    }
    *ms = best;
    return TBFS_OK;
  };
  /* every combination of a grid around the values that win on RMAT-like and
   * mesh-like graphs (coordinate search stalled in a local optimum there) */
  double cur = 0.0;
  st = time_of(a, b, pr, &cur);
  const float alphas[] = {4.0f, 6.0f, 9.0f, 12.0f, 15.0f, 24.0f, 60.0f};
  const float betas[] = {1.0f, 2.0f, 4.0f, 18.0f};
  const float ratios[] = {0.5f, 1.0f, 2.0f, 4.0f};
  const float a0 = a, b0 = b, p0 = pr;
  for (float xa : alphas)
    for (float xb : betas)
      for (float xp : ratios) {
        double t = 0.0;
        if (st != TBFS_OK || (xa == a0 && xb == b0 && xp == p0)) continue;
        if ((st = time_of(xa, xb, xp, &t)) == TBFS_OK && t < cur) {
          cur = t;
          a = xa;
          b = xb;
          pr = xp;
        }
      }
  tbfs::dev_free(S);
  tbfs::dev_free(sg);
  if (st != TBFS_OK) return st;
  opt->alpha = a;
  opt->beta = b;
  opt->pull_ratio = pr;
  tbfs::cache_store(cache_path, key, a, b, pr);
  return TBFS_OK;
}
