/*
 * graph_ingest.cu -- device-side preparation of a resident graph:
 *   validate_csc         bounds check of a CSC before any traversal reads it
 *   counting_sort_lists  (key, val) pairs -> ptr[n+1] / idx[nnz] lists; used
 *                        for COOC -> CSC (key = column) and for the transpose
 *                        CSC -> out-lists (key = row id)
 *   expand_columns       column id of every CSC entry
 *   symmetric_check      whether the CSC equals its transpose (keyed multiset hash)
 *   stable_sort_pairs    LSD radix sort of (key, val) pairs, 8 bits a pass,
 *                        stable: equal keys keep their input order
 * Replaces the host-side format builders of the reference
 * (TurboBFS_CSC_TD/sparseformatransf.c:28-120,
 * TurboBFS_COOC_TD/sparseformatransf.c:62-95) for graphs already on the GPU.
 * counting_sort_lists is stable too, so a list keeps the input order of its
 * entries: a COOC list the file order, a transposed list ascending columns.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
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

/* SplitMix64's output function (S. Vigna; a bijection of 64-bit words) */
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* Sum over the entries u -> v (u in column v) of h(u, v) - h(v, u), for two
 * keyed hashes h_k(x, y) = mix64(((x << 32) | y) ^ k), modulo 2^64.  A
 * warp takes chunks of kSymChunk consecutive entries; a lane follows its
 * entries' columns along col_ptr. */
constexpr int kSymChunk = 4096;
__global__ void symmetric_hash_kernel(const int *cp, const int *ic, int n, long long nnz,
                                      unsigned long long k1, unsigned long long k2,
                                      unsigned long long *out) {
  const unsigned lane = threadIdx.x & 31;
  const long long nchunks = (nnz + kSymChunk - 1) / kSymChunk;
  unsigned long long d1 = 0, d2 = 0;
  for (long long c = gtid() >> 5; c < nchunks; c += gstride() >> 5) {
    const long long e0 = c * kSymChunk;
    const long long e1 = e0 + kSymChunk < nnz ? e0 + kSymChunk : nnz;
    int col = (int)dev::warp_find_owner(cp, (unsigned)n, (unsigned)e0);
    for (long long k = e0 + lane; k < e1; k += 32) {
      while ((long long)__ldg(cp + col + 1) <= k) ++col;
      const unsigned long long u = (unsigned)__ldg(ic + k), v = (unsigned)col;
      const unsigned long long a = (u << 32) | v, b = (v << 32) | u;
      d1 += mix64(a ^ k1) - mix64(b ^ k1);
      d2 += mix64(a ^ k2) - mix64(b ^ k2);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    d2 += __shfl_xor_sync(0xffffffffu, d2, o);
  }
  if (lane == 0 && (d1 | d2)) {
    atomicAdd(out, d1);
    atomicAdd(out + 1, d2);
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

/* ---- stable LSD radix sort of (key, val) pairs ----
 * A pass sorts by the 8-bit digit (key >> shift) & 255.  Tiles of kRadixTile
 * consecutive pairs; hist[d * ntiles + t] counts digit d in tile t, and its
 * exclusive scan (digit-major) is where tile t's pairs of digit d start.
 * The scatter re-reads each tile in order -- warp w its 512-pair slice, 32
 * pairs a round -- and ranks equal digits by lane (match_any), so the output
 * keeps the input order among equal digits. */
constexpr int kRadixTile = 4096;
constexpr int kRadixWarpSlice = kRadixTile / (kThreads / 32);

__global__ void radix_hist_kernel(const unsigned *keys, long long len, int shift, int ntiles,
                                  int *hist) {
  __shared__ int h[256];
  for (int i = threadIdx.x; i < 256; i += kThreads) h[i] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRadixTile;
  for (int i = threadIdx.x; i < kRadixTile; i += kThreads) {
    const long long j = base + i;
    if (j < len) atomicAdd(&h[(keys[j] >> shift) & 255u], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kThreads) hist[(long long)d * ntiles + blockIdx.x] = h[d];
}

__global__ void radix_scatter_kernel(const unsigned *keys, const unsigned *vals, long long len,
                                     int shift, int ntiles, const int *offs, unsigned *ko,
                                     unsigned *vo) {
  static_assert(kThreads == 256, "one thread per digit in the warp prefix");
  __shared__ int cnt[kThreads / 32][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const long long base = (long long)blockIdx.x * kRadixTile + (long long)w * kRadixWarpSlice;
  for (int d = lane; d < 256; d += 32) cnt[w][d] = 0;
  __syncwarp();
  for (int r = 0; r < kRadixWarpSlice / 32; ++r) { /* digit counts of the warp's slice */
    const long long j = base + r * 32 + lane;
    const bool ok = j < len;
    const unsigned d = ok ? (keys[j] >> shift) & 255u : 256u + (unsigned)lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (ok && (peers & lt) == 0u) cnt[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  { /* start of each warp's digit d: the tile's start + earlier warps' counts */
    const int d = threadIdx.x;
    int run = offs[(long long)d * ntiles + blockIdx.x];
    for (int ww = 0; ww < kThreads / 32; ++ww) {
      const int c = cnt[ww][d];
      cnt[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int r = 0; r < kRadixWarpSlice / 32; ++r) {
    const long long j = base + r * 32 + lane;
    const bool ok = j < len;
    unsigned k = 0, v = 0;
    if (ok) {
      k = keys[j];
      v = vals[j];
    }
    const unsigned d = ok ? (k >> shift) & 255u : 256u + (unsigned)lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (ok) {
      const int pos = cnt[w][d] + __popc(peers & lt);
      ko[pos] = k;
      vo[pos] = v;
    }
    __syncwarp();
    if (ok && (peers & lt) == 0u) cnt[w][d] += __popc(peers);
    __syncwarp();
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

long long scan_partials(long long len) { return (len + kScanTile - 1) / kScanTile; }

/* exclusive scan over len ints with the caller's partial-sum scratch; queued
 * on s, no synchronisation */
cudaError_t exclusive_scan_ws(const int *in, long long len, int *out, int *partial,
                              cudaStream_t s) {
  const long long tiles = scan_partials(len);
  if (tiles == 0) return cudaSuccess;
  scan_reduce_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(in, len, partial);
  scan_partials_kernel<<<1, kThreads, 0, s>>>(partial, (int)tiles);
  scan_apply_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(in, len, partial, out);
  return cudaGetLastError();
}

/* exclusive scan over len ints, in place allowed; synchronises the stream */
cudaError_t exclusive_scan(const int *in, long long len, int *out, cudaStream_t s) {
  const long long tiles = scan_partials(len);
  if (tiles == 0) return cudaSuccess;
  int *partial = nullptr;
  cudaError_t e = tbfs::dev_alloc(&partial, (size_t)tiles * sizeof(int));
  if (e != cudaSuccess) return e;
  e = exclusive_scan_ws(in, len, out, partial, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  tbfs::dev_free(partial);
  return e != cudaSuccess ? e : e2;
}

cudaError_t validate_csc(const int *cp, const int *ic, int n, long long nnz, int *d_flag,
                         cudaStream_t s) {
  validate_kernel<<<grid_for(nnz > n ? nnz : n), kThreads, 0, s>>>(cp, ic, n, nnz, d_flag);
  return cudaGetLastError();
}

int key_bits(unsigned max_key) {
  int b = 0;
  while (b < 32 && (max_key >> b) != 0u) ++b;
  return b;
}

cudaError_t stable_sort_pairs(unsigned *keys, unsigned *vals, long long len, int bits,
                              unsigned *ktmp, unsigned *vtmp, cudaStream_t s) {
  if (len <= 1 || bits <= 0) return cudaSuccess;
  const long long tiles = (len + kRadixTile - 1) / kRadixTile;
  if (tiles * 256 > INT32_MAX) return cudaErrorInvalidValue;
  int *hist = nullptr;
  cudaError_t e = tbfs::dev_alloc(&hist, (size_t)tiles * 256 * sizeof(int));
  if (e != cudaSuccess) return e;
  unsigned *ka = keys, *va = vals, *kb = ktmp, *vb = vtmp;
  for (int shift = 0; shift < bits && e == cudaSuccess; shift += 8) {
    radix_hist_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(ka, len, shift, (int)tiles, hist);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = exclusive_scan(hist, tiles * 256, hist, s)) != cudaSuccess) break;
    radix_scatter_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(ka, va, len, shift, (int)tiles, hist,
                                                              kb, vb);
    e = cudaGetLastError();
    unsigned *t = ka;
    ka = kb;
    kb = t;
    t = va;
    va = vb;
    vb = t;
  }
  if (e == cudaSuccess && ka != keys) { /* odd number of passes: back to the caller's buffers */
    e = cudaMemcpyAsync(keys, ka, (size_t)len * sizeof(unsigned), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(vals, va, (size_t)len * sizeof(unsigned), cudaMemcpyDeviceToDevice, s);
  }
  cudaError_t e2 = cudaStreamSynchronize(s);
  tbfs::dev_free(hist);
  return e != cudaSuccess ? e : e2;
}

cudaError_t counting_sort_lists(const int *keys, const int *vals, long long nnz, int n,
                                int *ptr_out, int *idx_out, int *d_flag, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(ptr_out, 0, ((size_t)n + 1) * sizeof(int), s);
  if (e != cudaSuccess) return e;
  histogram_kernel<<<grid_for(nnz), kThreads, 0, s>>>(keys, nnz, n, ptr_out, d_flag);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan(ptr_out, (long long)n + 1, ptr_out, s)) != cudaSuccess) return e;
  int flag = 0;
  if ((e = cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  if (flag) return cudaSuccess; /* a key out of range: the caller reports it */
  /* stable: sort copies of the pairs by key, the values are the lists */
  const size_t m = (size_t)(nnz > 0 ? nnz : 1);
  unsigned *buf = nullptr;
  if ((e = tbfs::dev_alloc(&buf, 4 * m * sizeof(unsigned))) != cudaSuccess) return e;
  unsigned *k = buf, *v = buf + m, *kt = buf + 2 * m, *vt = buf + 3 * m;
  e = cudaMemcpyAsync(k, keys, (size_t)nnz * sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(v, vals, (size_t)nnz * sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = stable_sort_pairs(k, v, nnz, key_bits((unsigned)(n > 0 ? n - 1 : 0)), kt, vt, s);
  if (e == cudaSuccess && nnz)
    e = cudaMemcpyAsync(idx_out, v, (size_t)nnz * sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) { /* values out of range */
    validate_kernel<<<grid_for(nnz), kThreads, 0, s>>>(ptr_out, idx_out, n, nnz, d_flag);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamSynchronize(s);
  tbfs::dev_free(buf);
  return e != cudaSuccess ? e : e2;
}

cudaError_t symmetric_check(const int *cp, const int *ic, int n, long long nnz,
                            unsigned long long key1, unsigned long long key2, bool *symmetric,
                            cudaStream_t s) {
  *symmetric = false;
  unsigned long long *acc = nullptr, h[2] = {0, 0};
  cudaError_t e = tbfs::dev_alloc(&acc, 2 * sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), s);
  if (e == cudaSuccess && nnz > 0) {
    const long long warps = (nnz + kSymChunk - 1) / kSymChunk;
    const long long blocks = (warps * 32 + kThreads - 1) / kThreads;
    symmetric_hash_kernel<<<(unsigned)(blocks < 4864 ? blocks : 4864), kThreads, 0, s>>>(
        cp, ic, n, nnz, key1, key2, acc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  tbfs::dev_free(acc);
  if (e == cudaSuccess) *symmetric = h[0] == 0 && h[1] == 0;
  return e;
}

cudaError_t expand_columns(const int *cp, int n, int *col_of_entry, cudaStream_t s) {
  expand_kernel<<<grid_for((long long)n * 32), kThreads, 0, s>>>(cp, n, col_of_entry);
  return cudaGetLastError();
}

/* ---- degree-based grouping ----
 * Vertices are put into kGroups groups by degree relative to the mean
 * (group 0: degree < 2*mean; group g: 2^g*mean <= degree < 2^(g+1)*mean),
 * hottest group first, original order kept inside each group.  This is the
 * degree-based grouping of Faldu, Diamond and Grot (IISWC 2019): hubs end up
 * packed at the front, so the traversal's per-vertex gathers concentrate in
 * a few cache lines, while a graph without hubs keeps its layout (all its
 * vertices fall into group 0 and the order is the identity). */

namespace {

constexpr int kGroups = 16;
constexpr int kGroupTile = 1024; /* vertices per single-warp block */

__device__ __forceinline__ int degree_group(const int *cp, int v, float inv_mean2) {
  const float t = (float)(cp[v + 1] - cp[v]) * inv_mean2; /* degree / (2*mean) */
  if (t < 1.0f) return 0;
  const int g = 1 + (int)floorf(log2f(t));
  return g < kGroups - 1 ? g : kGroups - 1;
}

/* counts[slot(g, b)] with slot = (kGroups-1-g) * nblocks + b */
__global__ void group_count_kernel(const int *cp, int n, float inv_mean2, int *counts) {
  __shared__ int c[kGroups];
  const int lane = threadIdx.x;
  if (lane < kGroups) c[lane] = 0;
  __syncwarp();
  const long long base = (long long)blockIdx.x * kGroupTile;
  for (int i = lane; i < kGroupTile; i += 32) {
    const long long v = base + i;
    if (v < n) atomicAdd(&c[degree_group(cp, (int)v, inv_mean2)], 1);
  }
  __syncwarp();
  if (lane < kGroups) counts[(size_t)(kGroups - 1 - lane) * gridDim.x + blockIdx.x] = c[lane];
}

/* stable scatter: one warp walks its tile in order, ranking equal groups
 * with __match_any_sync */
__global__ void group_scatter_kernel(const int *cp, int n, float inv_mean2, const int *offsets,
                                     int *perm, int *inv) {
  __shared__ int off[kGroups + 1];
  const int lane = threadIdx.x;
  if (lane < kGroups) off[lane] = offsets[(size_t)(kGroups - 1 - lane) * gridDim.x + blockIdx.x];
  __syncwarp();
  const long long base = (long long)blockIdx.x * kGroupTile;
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  for (int c0 = 0; c0 < kGroupTile; c0 += 32) {
    const long long v = base + c0 + lane;
    const int g = v < n ? degree_group(cp, (int)v, inv_mean2) : kGroups;
    const unsigned m = __match_any_sync(0xffffffffu, g);
    const int rank = __popc(m & lt);
    if (g < kGroups) {
      const int pos = off[g] + rank;
      perm[pos] = (int)v;
      inv[v] = pos;
    }
    __syncwarp();
    if (g < kGroups && (m >> lane) == 1u) off[g] += __popc(m); /* last lane of its group */
    __syncwarp();
  }
}

__global__ void permuted_degree_kernel(const int *cp, const int *perm, int n, int *deg2) {
  for (unsigned long long i = gtid(); i < (unsigned long long)n; i += gstride()) {
    const int v = perm[i];
    deg2[i] = cp[v + 1] - cp[v];
  }
}

/* one warp per new column i copies old column perm[i], renaming its rows */
/* New list i is old list perm[i] with every entry renamed by inv, in the same
 * order.  Short lists (< 32 entries) are copied by one lane each; long ones
 * are collected into `longs` (count in longs[-1] ... see below) and copied by
 * a block each, so that a hub's list is spread over 256 threads. */
__global__ void permuted_short_lists_kernel(const int *cp, const int *ic, const int *perm,
                                            const int *inv, const int *cp2, int n, int *ic2,
                                            int *longs, int *nlong) {
  const unsigned lane = threadIdx.x & 31;
  for (unsigned long long base = gtid() & ~31ull; base < (unsigned long long)n; base += gstride()) {
    const unsigned long long i = base + lane;
    int b = 0, len = 0, o = 0;
    if (i < (unsigned long long)n) {
      const int v = perm[i];
      b = cp[v];
      len = cp[v + 1] - b;
      o = cp2[i];
    }
    if (len < 32)
      for (int t = 0; t < len; ++t) ic2[o + t] = inv[ic[b + t]];
    /* append the long ones, one atomic per warp */
    const bool lng = len >= 32;
    const unsigned bal = __ballot_sync(0xffffffffu, lng);
    if (bal) {
      int pos = 0;
      if (lane == 0) pos = atomicAdd(nlong, __popc(bal));
      pos = __shfl_sync(0xffffffffu, pos, 0);
      if (lng) longs[pos + __popc(bal & ((1u << lane) - 1u))] = (int)i;
    }
  }
}

__global__ void permuted_long_lists_kernel(const int *cp, const int *ic, const int *perm,
                                           const int *inv, const int *cp2, const int *longs,
                                           const int *nlong, int *ic2) {
  const int cnt = *nlong;
  for (int j = blockIdx.x; j < cnt; j += gridDim.x) {
    const int i = longs[j];
    const int v = perm[i];
    const int b = cp[v], len = cp[v + 1] - b, o = cp2[i];
    for (int t = threadIdx.x; t < len; t += blockDim.x) ic2[o + t] = inv[ic[b + t]];
  }
}

}  // namespace

cudaError_t degree_group_relabel(const int *cp, const int *ic, int n, long long nnz,
                                 int *perm, int *inv, int *cp2, int *ic2, bool *identity,
                                 cudaStream_t s) {
  const int nblocks = (int)((n + (long long)kGroupTile - 1) / kGroupTile);
  const float inv_mean2 = nnz > 0 ? (float)((double)n / (2.0 * (double)nnz)) : 0.0f;
  int *counts = nullptr;
  const size_t nslots = (size_t)kGroups * nblocks;
  cudaError_t e = tbfs::dev_alloc(&counts, (nslots + 1) * sizeof(int));
  if (e != cudaSuccess) return e;
  group_count_kernel<<<nblocks, 32, 0, s>>>(cp, n, inv_mean2, counts);
  e = cudaGetLastError();
  /* how many vertices sit outside group 0: if none, the order is the identity */
  int tail_first = 0;
  if (e == cudaSuccess)
    e = exclusive_scan(counts, (long long)nslots + 1, counts, s);
  if (e == cudaSuccess)
    e = cudaMemcpy(&tail_first, counts + (size_t)(kGroups - 1) * nblocks, sizeof(int),
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) {
    *identity = tail_first == 0;
    if (!*identity) {
      group_scatter_kernel<<<nblocks, 32, 0, s>>>(cp, n, inv_mean2, counts, perm, inv);
      permuted_degree_kernel<<<grid_for(n), kThreads, 0, s>>>(cp, perm, n, cp2);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaMemsetAsync(cp2 + n, 0, sizeof(int), s);
      if (e == cudaSuccess) e = exclusive_scan(cp2, (long long)n + 1, cp2, s);
      int *longs = nullptr; /* long lists' new ids, their count after them */
      if (e == cudaSuccess) e = tbfs::dev_alloc(&longs, ((size_t)n + 1) * sizeof(int));
      if (e == cudaSuccess) e = cudaMemsetAsync(longs + n, 0, sizeof(int), s);
      if (e == cudaSuccess) {
        permuted_short_lists_kernel<<<grid_for(n), kThreads, 0, s>>>(cp, ic, perm, inv, cp2, n,
                                                                    ic2, longs, longs + n);
        permuted_long_lists_kernel<<<4096, kThreads, 0, s>>>(cp, ic, perm, inv, cp2, longs,
                                                             longs + n, ic2);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      tbfs::dev_free(longs);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
  }
  tbfs::dev_free(counts);
  return e;
}

}  // namespace tbfs
