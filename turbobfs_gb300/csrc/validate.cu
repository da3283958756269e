/*
 * validate.cu -- check a BFS result against the graph on the device
 * (tbfs_bfs_validate).
 *
 * The reference checks its GPU result by comparing it with its own
 * sequential BFS (S_check / bfs_check, TurboBFS_CSC_TD/utils_bfs.c:93-145),
 * which costs a second traversal on the host.  Here a result is checked
 * against the graph itself, in the manner of the Graph500 validation step:
 * S and sigma are the unique depth and path-count vectors of (graph, root)
 * exactly when
 *   - S[root] = 0, sigma[root] = 1, and no other vertex is at depth 0;
 *   - every edge u->v out of a reached u reaches v with S[v] <= S[u] + 1;
 *   - every reached v != root has an in-neighbour at depth S[v] - 1;
 *   - sigma[v] = sum of sigma[u] over the in-list entries u at depth
 *     S[v] - 1 (mod 2^64, the engine's wrap-around arithmetic), and 0 for
 *     unreached vertices.
 * One pass over the in-lists: a lane per vertex for lists of up to kHeavy
 * entries, a block per longer list (collected by the first pass).  Every
 * violation is counted by kind, with the smallest offending vertex.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "tbfs.h"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

constexpr int kHeavy = 128;
constexpr int kThreads = 256;

enum { V_ROOT = 0, V_DEPTH, V_SKIP, V_PARENT, V_SIGMA, V_VISITED, V_EDGES, V_NHEAVY, V_COUNT };

struct VCounters {
  unsigned long long c[V_COUNT];
  int first_bad; /* smallest caller id with a violation (INT_MAX: none) */
};

struct VParams {
  const int *cp, *ic;
  const int *perm; /* internal id -> caller id, or null */
  int n, root;     /* root: caller numbering */
  const int *S;
  const unsigned long long *sigma; /* null: depths only */
  int *heavy;      /* internal ids of lists longer than kHeavy */
  VCounters *out;
};

/* the per-vertex checks, once the list's contribution is known; returns
 * the counts to add (bit per kind) */
__device__ __forceinline__ unsigned vertex_verdict(const VParams &p, int v, int Sv, bool has_parent,
                                                   unsigned long long sum) {
  unsigned bad = 0;
  if (Sv < -1) bad |= 1u << V_DEPTH;
  if (v == p.root) {
    if (Sv != 0 || (p.sigma && p.sigma[v] != 1ull)) bad |= 1u << V_ROOT;
  } else if (Sv == 0) {
    bad |= 1u << V_ROOT;
  } else if (Sv > 0) {
    if (!has_parent) bad |= 1u << V_PARENT;
    if (p.sigma && p.sigma[v] != sum) bad |= 1u << V_SIGMA;
  } else if (p.sigma && p.sigma[v] != 0ull) {
    bad |= 1u << V_SIGMA;
  }
  return bad;
}

/* one entry u -> v: updates the skip count, parent flag and parent sum */
__device__ __forceinline__ void entry_check(const VParams &p, int Sv, int u_int, unsigned &skips,
                                            bool &has_parent, unsigned long long &sum) {
  const int u = p.perm ? __ldg(p.perm + u_int) : u_int;
  const int Su = p.S[u];
  if (Su < 0) return;
  if (Sv < 0 || Sv > Su + 1) ++skips;
  if (Su == Sv - 1) {
    has_parent = true;
    if (p.sigma) sum += p.sigma[u];
  }
}

__device__ __forceinline__ void add_counts(VCounters *out, unsigned bad, unsigned skips,
                                           unsigned visited, unsigned long long edges, int v) {
  /* warp-aggregated: counts of this lane, summed over the warp */
  unsigned long long cnt[V_NHEAVY];
#pragma unroll
  for (int k = 0; k < V_NHEAVY; ++k) cnt[k] = 0;
#pragma unroll
  for (int k = 0; k < V_VISITED; ++k) cnt[k] = (bad >> k) & 1u;
  cnt[V_SKIP] = skips;
  cnt[V_VISITED] = visited;
  cnt[V_EDGES] = edges;
#pragma unroll
  for (int k = 0; k < V_NHEAVY; ++k)
    for (int o = 16; o > 0; o >>= 1) cnt[k] += __shfl_xor_sync(0xffffffffu, cnt[k], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < V_NHEAVY; ++k)
      if (cnt[k]) atomicAdd(&out->c[k], cnt[k]);
  if (bad || skips) atomicMin(&out->first_bad, v);
}

__global__ void __launch_bounds__(kThreads) validate_light_kernel(VParams p) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n_round = ((long long)p.n + 31) / 32 * 32; /* whole warps in every round */
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
    unsigned bad = 0, skips = 0, visited = 0;
    unsigned long long edges = 0;
    int v = 0x7fffffff;
    bool heavy = false;
    if (i < p.n) {
      v = p.perm ? __ldg(p.perm + i) : (int)i;
      const int Sv = p.S[v];
      const int b = __ldg(p.cp + i), e = __ldg(p.cp + i + 1);
      if (e - b > kHeavy) {
        heavy = true;
      } else {
        bool has_parent = false;
        unsigned long long sum = 0;
        for (int k = b; k < e; ++k) entry_check(p, Sv, __ldg(p.ic + k), skips, has_parent, sum);
        bad = vertex_verdict(p, v, Sv, has_parent, sum);
        visited = Sv >= 0;
        edges = Sv >= 0 ? (unsigned long long)(e - b) : 0ull;
      }
    }
    const unsigned hb = __ballot_sync(0xffffffffu, heavy);
    if (hb) {
      unsigned long long pos = 0;
      if ((threadIdx.x & 31) == 0) pos = atomicAdd(&p.out->c[V_NHEAVY], (unsigned long long)__popc(hb));
      pos = __shfl_sync(0xffffffffu, pos, 0);
      if (heavy) p.heavy[pos + __popc(hb & ((1u << (threadIdx.x & 31)) - 1u))] = (int)i;
    }
    add_counts(p.out, bad, skips, visited, edges, v);
  }
}

/* a block per long list: the entries strided over the block, reduced */
__global__ void __launch_bounds__(kThreads) validate_heavy_kernel(VParams p) {
  __shared__ unsigned s_skips, s_parent;
  __shared__ unsigned long long s_sum;
  const unsigned long long nh = p.out->c[V_NHEAVY];
  for (unsigned long long j = blockIdx.x; j < nh; j += gridDim.x) {
    const int i = p.heavy[j];
    const int v = p.perm ? __ldg(p.perm + i) : i;
    const int Sv = p.S[v];
    const int b = __ldg(p.cp + i), e = __ldg(p.cp + i + 1);
    if (threadIdx.x == 0) {
      s_skips = 0;
      s_parent = 0;
      s_sum = 0;
    }
    __syncthreads();
    unsigned skips = 0;
    bool has_parent = false;
    unsigned long long sum = 0;
    for (int k = b + (int)threadIdx.x; k < e; k += blockDim.x)
      entry_check(p, Sv, __ldg(p.ic + k), skips, has_parent, sum);
    for (int o = 16; o > 0; o >>= 1) {
      skips += __shfl_xor_sync(0xffffffffu, skips, o);
      sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    const bool any_parent = __any_sync(0xffffffffu, has_parent);
    if ((threadIdx.x & 31) == 0) {
      if (skips) atomicAdd(&s_skips, skips);
      if (any_parent) s_parent = 1u;
      if (sum) atomicAdd(&s_sum, sum);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      unsigned bad = 0, sk = 0, vis = 0;
      unsigned long long ed = 0;
      if (threadIdx.x == 0) {
        bad = vertex_verdict(p, v, Sv, s_parent != 0, s_sum);
        sk = s_skips;
        vis = Sv >= 0;
        ed = Sv >= 0 ? (unsigned long long)(e - b) : 0ull;
      }
      add_counts(p.out, bad, sk, vis, ed, threadIdx.x == 0 ? v : 0x7fffffff);
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace tbfs

extern "C" tbfs_status tbfs_bfs_validate(tbfs_graph *g, int32_t root, const int32_t *S,
                                         const int64_t *sigma, int32_t on_device, void *stream,
                                         tbfs_validation *out) {
  if (!g || !S || !out) {
    tbfs_set_error("tbfs_bfs_validate: null graph, depth vector or result");
    return TBFS_ERR_INVALID_ARG;
  }
  if (root < 0 || root >= g->n) {
    tbfs_set_error("tbfs_bfs_validate: root %d outside [0, %d)", root, g->n);
    return TBFS_ERR_INVALID_ARG;
  }
  memset(out, 0, sizeof *out);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)g->n;
  /* one scratch block: counters, heavy list, and the host inputs' copies */
  size_t off_heavy = (sizeof(tbfs::VCounters) + 255) / 256 * 256;
  size_t off_S = off_heavy + (n * sizeof(int) + 255) / 256 * 256;
  size_t off_sg = off_S + (on_device ? 0 : (n * sizeof(int) + 255) / 256 * 256);
  size_t total = off_sg + (on_device || !sigma ? 0 : n * sizeof(unsigned long long));
  char *scratch = nullptr;
  cudaError_t e = cudaSetDevice(g->device);
  if (e == cudaSuccess) e = tbfs::dev_alloc(&scratch, total);
  tbfs::VParams p = {};
  tbfs::VCounters hc = {};
  if (e == cudaSuccess) {
    p.cp = g->cp;
    p.ic = g->ic;
    p.perm = g->perm;
    p.n = g->n;
    p.root = root;
    p.out = reinterpret_cast<tbfs::VCounters *>(scratch);
    p.heavy = reinterpret_cast<int *>(scratch + off_heavy);
    if (on_device) {
      p.S = S;
      p.sigma = reinterpret_cast<const unsigned long long *>(sigma);
    } else {
      int *dS = reinterpret_cast<int *>(scratch + off_S);
      e = cudaMemcpyAsync(dS, S, n * sizeof(int), cudaMemcpyHostToDevice, s);
      p.S = dS;
      if (e == cudaSuccess && sigma) {
        unsigned long long *dsg = reinterpret_cast<unsigned long long *>(scratch + off_sg);
        e = cudaMemcpyAsync(dsg, sigma, n * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
        p.sigma = dsg;
      }
    }
  }
  if (e == cudaSuccess) {
    hc.first_bad = 0x7fffffff;
    e = cudaMemcpyAsync(p.out, &hc, sizeof hc, cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess) {
    const int blocks = (int)(((long long)g->n + tbfs::kThreads - 1) / tbfs::kThreads < 4864
                                 ? ((long long)g->n + tbfs::kThreads - 1) / tbfs::kThreads
                                 : 4864);
    tbfs::validate_light_kernel<<<blocks > 0 ? blocks : 1, tbfs::kThreads, 0, s>>>(p);
    tbfs::validate_heavy_kernel<<<1216, tbfs::kThreads, 0, s>>>(p);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, p.out, sizeof hc, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  tbfs::dev_free(scratch);
  if (e != cudaSuccess) {
    tbfs_set_error("tbfs_bfs_validate: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TBFS_ERR_OUT_OF_MEMORY : TBFS_ERR_CUDA;
  }
  out->bad_root = (int64_t)hc.c[tbfs::V_ROOT];
  out->bad_depth = (int64_t)hc.c[tbfs::V_DEPTH];
  out->skips_level = (int64_t)hc.c[tbfs::V_SKIP];
  out->no_parent = (int64_t)hc.c[tbfs::V_PARENT];
  out->sigma_mismatch = (int64_t)hc.c[tbfs::V_SIGMA];
  out->visited = (int64_t)hc.c[tbfs::V_VISITED];
  out->edges = (int64_t)hc.c[tbfs::V_EDGES];
  out->first_bad = hc.first_bad == 0x7fffffff ? -1 : hc.first_bad;
  return TBFS_OK;
}
