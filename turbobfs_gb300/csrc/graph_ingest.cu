/*
 * graph_ingest.cu -- device-side preparation of a resident graph:
 *   validate_csc         bounds check of a CSC before any traversal reads it
 *   counting_sort_lists  (key, val) pairs -> ptr[n+1] / idx[nnz] lists; used
 *                        for COOC -> CSC (key = column) and for the transpose
 *                        CSC -> out-lists (key = row id)
 *   expand_columns       column id of every CSC entry
 * Replaces the host-side format builders of the reference
 * (TurboBFS_CSC_TD/sparseformatransf.c:28-120,
 * TurboBFS_COOC_TD/sparseformatransf.c:62-95) for graphs already on the GPU.
 * The order of entries inside a list after counting_sort_lists is not
 * deterministic; BFS depth and path counts do not depend on it.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "tbfs_internal.h"

namespace tbfs {
namespace {

constexpr int kThreads = 256;
constexpr int kScanTile = 4096; /* elements per block in the scan passes */

__device__ __forceinline__ unsigned long long gtid() {
  return (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ unsigned long long gstride() {
  return (unsigned long long)gridDim.x * blockDim.x;
}

/* flag bit 1: col_ptr malformed; bit 2: row id out of range */
__global__ void validate_kernel(const int *cp, const int *ic, int n, long long nnz,
                                int *flag) {
  for (unsigned long long v = gtid(); v < (unsigned long long)n; v += gstride())
    if (cp[v] > cp[v + 1]) atomicOr(flag, 1);
  if (gtid() == 0 && (cp[0] != 0 || (long long)cp[n] != nnz)) atomicOr(flag, 1);
  for (unsigned long long k = gtid(); k < (unsigned long long)nnz; k += gstride()) {
    const int u = ic[k];
    if (u < 0 || u >= n) atomicOr(flag, 2);
  }
}

__global__ void histogram_kernel(const int *keys, long long nnz, int n, int *cnt,
                                 int *flag) {
  for (unsigned long long k = gtid(); k < (unsigned long long)nnz; k += gstride()) {
    const int key = keys[k];
    if (key < 0 || key >= n) {
      atomicOr(flag, 2);
      continue;
    }
    atomicAdd(cnt + key, 1);
  }
}

__global__ void scatter_kernel(const int *keys, const int *vals, long long nnz, int n,
                               int *fill, int *idx, int *flag) {
  for (unsigned long long k = gtid(); k < (unsigned long long)nnz; k += gstride()) {
    const int key = keys[k], val = vals[k];
    if (key < 0 || key >= n || val < 0 || val >= n) {
      atomicOr(flag, 2);
      continue;
    }
    const int pos = atomicAdd(fill + key, 1);
    idx[pos] = val;
  }
}

/* one warp per column writes the column id over its entry range */
__global__ void expand_kernel(const int *cp, int n, int *col) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned long long w0 = gtid() >> 5, nw = gstride() >> 5;
  for (unsigned long long v = w0; v < (unsigned long long)n; v += nw) {
    const int b = cp[v], e = cp[v + 1];
    for (int k = b + (int)lane; k < e; k += 32) col[k] = (int)v;
  }
}

/* ---- exclusive scan of int32 counts (three passes) ---- */

__device__ int block_excl_scan(int x, int *smem, int *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) smem[w] = incl;
  __syncthreads();
  if (w == 0) {
    int v = lane < (kThreads / 32) ? smem[lane] : 0;
    int vi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, vi, o);
      if (lane >= o) vi += t;
    }
    if (lane < (kThreads / 32)) smem[lane] = vi - v;
    if (lane == 31) smem[32] = vi;
  }
  __syncthreads();
  const int r = incl - x + smem[w];
  *total = smem[32];
  __syncthreads();
  return r;
}

__global__ void scan_reduce_kernel(const int *in, long long len, int *partial) {
  __shared__ int smem[33];
  const long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += kThreads) {
    const long long j = base + i;
    if (j < len) s += in[j];
  }
  int total;
  block_excl_scan(s, smem, &total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void scan_partials_kernel(int *partial, int nparts) {
  __shared__ int smem[33];
  int carry = 0;
  for (int b0 = 0; b0 < nparts; b0 += kThreads) {
    const int i = b0 + threadIdx.x;
    const int x = i < nparts ? partial[i] : 0;
    int total;
    const int ex = block_excl_scan(x, smem, &total);
    if (i < nparts) partial[i] = ex + carry;
    carry += total;
  }
}

/* out[j] = exclusive prefix of in[] (in and out may alias) */
__global__ void scan_apply_kernel(const int *in, long long len, const int *partial,
                                  int *out) {
  __shared__ int smem[33];
  const long long base = (long long)blockIdx.x * kScanTile;
  int carry = partial[blockIdx.x];
  constexpr int kPer = kScanTile / kThreads;
  /* each thread owns kPer consecutive elements */
  int vals[kPer];
  int s = 0;
  const long long mine = base + (long long)threadIdx.x * kPer;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    vals[i] = (mine + i < len) ? in[mine + i] : 0;
    s += vals[i];
  }
  int total;
  int ex = block_excl_scan(s, smem, &total) + carry;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    if (mine + i < len) out[mine + i] = ex;
    ex += vals[i];
  }
}

int grid_for(long long work) {
  long long g = (work + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (g > 65535LL * 8) g = 65535LL * 8;
  return (int)g;
}

}  // namespace

/* exclusive scan over len ints, in place allowed */
static cudaError_t exclusive_scan(const int *in, long long len, int *out, cudaStream_t s) {
  const long long tiles = (len + kScanTile - 1) / kScanTile;
  if (tiles == 0) return cudaSuccess;
  int *partial = nullptr;
  cudaError_t e = cudaMalloc(&partial, (size_t)tiles * sizeof(int));
  if (e != cudaSuccess) return e;
  scan_reduce_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(in, len, partial);
  scan_partials_kernel<<<1, kThreads, 0, s>>>(partial, (int)tiles);
  scan_apply_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(in, len, partial, out);
  e = cudaGetLastError();
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(partial);
  return e != cudaSuccess ? e : e2;
}

cudaError_t validate_csc(const int *cp, const int *ic, int n, long long nnz, int *d_flag,
                         cudaStream_t s) {
  validate_kernel<<<grid_for(nnz > n ? nnz : n), kThreads, 0, s>>>(cp, ic, n, nnz, d_flag);
  return cudaGetLastError();
}

cudaError_t counting_sort_lists(const int *keys, const int *vals, long long nnz, int n,
                                int *ptr_out, int *idx_out, int *d_flag, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(ptr_out, 0, ((size_t)n + 1) * sizeof(int), s);
  if (e != cudaSuccess) return e;
  histogram_kernel<<<grid_for(nnz), kThreads, 0, s>>>(keys, nnz, n, ptr_out, d_flag);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan(ptr_out, (long long)n + 1, ptr_out, s)) != cudaSuccess) return e;
  int *fill = nullptr;
  if ((e = cudaMalloc(&fill, ((size_t)n + 1) * sizeof(int))) != cudaSuccess) return e;
  e = cudaMemcpyAsync(fill, ptr_out, ((size_t)n + 1) * sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) {
    scatter_kernel<<<grid_for(nnz), kThreads, 0, s>>>(keys, vals, nnz, n, fill, idx_out, d_flag);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(fill);
  return e != cudaSuccess ? e : e2;
}

cudaError_t expand_columns(const int *cp, int n, int *col_of_entry, cudaStream_t s) {
  expand_kernel<<<grid_for((long long)n * 32), kThreads, 0, s>>>(cp, n, col_of_entry);
  return cudaGetLastError();
}

}  // namespace tbfs
