/*
 * mm_ingest.cu -- graphs built on the device from edge lists and from
 * Matrix Market text.
 *
 *   csc_from_edges_device  edge list (on the device) -> CSC, with the
 *                          construction of the host builder
 *                          tbfs_csc_from_edges: symmetrise (each entry and
 *                          its mirror, a self loop twice), drop self loops,
 *                          sort each column, drop repeats.  Built by stable
 *                          radix sorts, so without sorting a column keeps the
 *                          input order of its entries, exactly as the host
 *                          builder lays it out.
 *   mm_parse_device        the data lines of a Matrix Market coordinate
 *                          file (already in device memory) -> edge list,
 *                          entry k from the k-th data line.
 *
 * These replace the reference's host preparation -- readMMfile_uw and the
 * CP_RP_ug / SSCCSC_uw / SSCCOOC_uw builders
 * (TurboBFS_CSC_TD/readMMfilef.c:56-70, TurboBFS_CSC_TD/sparseformatransf.c:
 * 60-104, TurboBFS_COOC_TD/sparseformatransf.c:62-95) -- which the host
 * reader tbfs_mm_read restates sequentially.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "tbfs_graphgen.h"
#include "tbfs_internal.h"

namespace tbfs {
namespace {

constexpr int kThreads = 256;
constexpr int kTextPer = 16;                       /* bytes a thread looks at */
constexpr int kTextTile = kThreads * kTextPer;     /* bytes a block looks at  */

__device__ __forceinline__ unsigned long long gtid() {
  return (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ unsigned long long gstride() {
  return (unsigned long long)gridDim.x * blockDim.x;
}

int grid_for(long long work) {
  long long g = (work + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (g > 65535LL * 8) g = 65535LL * 8;
  return (int)g;
}

/* ---- edge list -> CSC ---- */

/* entry e of the pair list: (column, row); with symmetrise edge k gives
 * e = 2k (dst <- src) and e = 2k+1 (src <- dst).  Dropped or invalid edges
 * get column n, which sorts last and is cut off. */
__global__ void edge_pairs_kernel(const int *src, const int *dst, long long m, int n,
                                  unsigned flags, unsigned *key, unsigned *val, int *bad) {
  const bool sym = (flags & TBFS_BUILD_SYMMETRIZE) != 0u;
  const bool noloop = (flags & TBFS_BUILD_DROP_LOOPS) != 0u;
  for (unsigned long long k = gtid(); k < (unsigned long long)m; k += gstride()) {
    const int u = src[k], v = dst[k];
    const bool ok = u >= 0 && u < n && v >= 0 && v < n;
    if (!ok) atomicOr(bad, 1);
    const bool drop = !ok || (noloop && u == v);
    const unsigned long long e = sym ? 2 * k : k;
    key[e] = drop ? (unsigned)n : (unsigned)v;
    val[e] = ok ? (unsigned)u : 0u;
    if (sym) {
      key[e + 1] = drop ? (unsigned)n : (unsigned)u;
      val[e + 1] = ok ? (unsigned)v : 0u;
    }
  }
}

/* keep[i] = pair i is a real entry (column < n) and, with dedup, differs
 * from pair i-1 (the pairs are sorted by column, then row) */
__global__ void keep_kernel(const unsigned *key, const unsigned *val, long long len, int n,
                            int dedup, int *keep) {
  for (unsigned long long i = gtid(); i < (unsigned long long)len; i += gstride()) {
    int k = key[i] < (unsigned)n ? 1 : 0;
    if (k && dedup && i > 0 && key[i] == key[i - 1] && val[i] == val[i - 1]) k = 0;
    keep[i] = k;
  }
}

/* cnt[key] += kept pairs; the keys are sorted, so a warp's lanes mostly
 * share one: one atomic per distinct key of the warp (match_any) */
__global__ void column_count_kernel(const unsigned *key, const int *keep, long long len, int *cnt) {
  const int lane = threadIdx.x & 31;
  for (unsigned long long i = gtid(); i < (unsigned long long)len; i += gstride()) {
    const unsigned act = __activemask();
    const unsigned k = keep[i] ? key[i] : 0xffffffffu;
    const unsigned peers = __match_any_sync(act, k);
    if (k != 0xffffffffu && (peers & ((1u << lane) - 1u)) == 0u)
      atomicAdd(cnt + k, __popc(peers));
  }
}

/* rows of the kept pairs at their compacted positions (keep scanned) */
__global__ void compact_kernel(const unsigned *val, const int *keep_flag, const int *pos,
                               long long len, int *ic) {
  for (unsigned long long i = gtid(); i < (unsigned long long)len; i += gstride())
    if (keep_flag[i]) ic[pos[i]] = (int)val[i];
}

/* ---- Matrix Market data lines -> edge list ---- */

__device__ __forceinline__ bool blank(char c) { return c == ' ' || c == '\t' || c == '\r'; }
__device__ __forceinline__ bool digit(char c) { return c >= '0' && c <= '9'; }

/* p starts a data line: the first byte of a line whose first non-blank
 * byte is a digit (comment lines start with '%', empty lines have none) */
__device__ __forceinline__ bool entry_start(const char *t, long long len, long long p) {
  if (p >= len || (p > 0 && t[p - 1] != '\n')) return false;
  long long q = p;
  while (q < len && blank(t[q])) ++q;
  return q < len && digit(t[q]);
}

__device__ int block_excl_sum(int x, int *smem, int *total) {
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
    const int v = lane < kThreads / 32 ? smem[lane] : 0;
    int vi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, vi, o);
      if (lane >= o) vi += t;
    }
    if (lane < kThreads / 32) smem[lane] = vi - v;
    if (lane == 31) smem[32] = vi;
  }
  __syncthreads();
  const int r = incl - x + smem[w];
  *total = smem[32];
  __syncthreads();
  return r;
}

/* counts[tile] = data lines starting in the tile's kTextTile bytes */
__global__ void mm_count_kernel(const char *t, long long len, int *counts) {
  __shared__ int smem[33];
  const long long p0 = (long long)blockIdx.x * kTextTile + (long long)threadIdx.x * kTextPer;
  int c = 0;
#pragma unroll 4
  for (int i = 0; i < kTextPer; ++i) c += entry_start(t, len, p0 + i) ? 1 : 0;
  int total;
  block_excl_sum(c, smem, &total);
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

/* reads the unsigned decimal at t[*q..), advancing *q; false without digits
 * or past 2^40 (far beyond any int32 index) */
__device__ bool read_uint(const char *t, long long len, long long *q, unsigned long long *x) {
  long long r = *q;
  unsigned long long v = 0;
  int nd = 0;
  while (r < len && digit(t[r])) {
    v = v * 10u + (unsigned long long)(t[r] - '0');
    if (v > (1ull << 40)) return false;
    ++r;
    ++nd;
  }
  *q = r;
  *x = v;
  return nd > 0;
}

/* Entry k (the k-th data line, k < nz): row i and column j, 1-based, as the
 * edge i-1 -> j-1.  A line that does not hold two indices with 1 <= i <= M,
 * 1 <= j <= N and i <= N records its k in *bad (the smallest wins). */
__global__ void mm_parse_kernel(const char *t, long long len, const int *offs, long long nz,
                                long long M, long long N, int *src, int *dst,
                                unsigned long long *bad) {
  __shared__ int smem[33];
  const long long p0 = (long long)blockIdx.x * kTextTile + (long long)threadIdx.x * kTextPer;
  unsigned starts = 0; /* bit i: p0 + i starts a data line */
#pragma unroll 4
  for (int i = 0; i < kTextPer; ++i)
    if (entry_start(t, len, p0 + i)) starts |= 1u << i;
  int total;
  long long k = (long long)offs[blockIdx.x] + block_excl_sum(__popc(starts), smem, &total);
  while (starts) {
    const int i = __ffs(starts) - 1;
    starts &= starts - 1u;
    if (k < nz) {
      long long q = p0 + i;
      while (q < len && blank(t[q])) ++q;
      unsigned long long a = 0, b = 0;
      bool ok = read_uint(t, len, &q, &a);
      if (ok) {
        const long long q0 = q;
        while (q < len && blank(t[q])) ++q;
        ok = q > q0 && read_uint(t, len, &q, &b);
      }
      ok = ok && a >= 1 && b >= 1 && (long long)a <= M && (long long)b <= N && (long long)a <= N;
      if (ok) {
        src[k] = (int)(a - 1);
        dst[k] = (int)(b - 1);
      } else {
        atomicMin(bad, (unsigned long long)k);
        src[k] = 0;
        dst[k] = 0;
      }
    }
    ++k;
  }
}

}  // namespace

cudaError_t csc_from_edges_device(const int *src, const int *dst, long long m, int n,
                                  unsigned flags, int **cp_out, int **ic_out, long long *nnz_out,
                                  int *bad_out, cudaStream_t s) {
  *cp_out = nullptr;
  *ic_out = nullptr;
  *nnz_out = 0;
  *bad_out = 0;
  const bool sym = (flags & TBFS_BUILD_SYMMETRIZE) != 0u;
  const bool dedup = (flags & TBFS_BUILD_DEDUP) != 0u;
  const bool sorted = dedup || (flags & TBFS_BUILD_SORT) != 0u;
  const long long len = sym ? 2 * m : m;
  if (len > INT32_MAX) return cudaErrorInvalidValue;
  const size_t L = (size_t)(len > 0 ? len : 1);
  unsigned *buf = nullptr;
  int *cnt = nullptr, *keep = nullptr, *dflag = nullptr, *cp = nullptr, *ic = nullptr;
  cudaError_t e = tbfs::dev_alloc(&buf, 4 * L * sizeof(unsigned));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&keep, (L + 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&dflag, sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&cp, ((size_t)n + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(dflag, 0, sizeof(int), s);
  unsigned *key = buf, *val = buf + L, *kt = buf + 2 * L, *vt = buf + 3 * L;
  if (e == cudaSuccess && m > 0) {
    edge_pairs_kernel<<<grid_for(m), kThreads, 0, s>>>(src, dst, m, n, flags, key, val, dflag);
    e = cudaGetLastError();
  }
  /* rows ascending inside a column: sort by row first, then (stably) by column */
  if (e == cudaSuccess && sorted)
    e = stable_sort_pairs(val, key, len, key_bits((unsigned)(n - 1)), vt, kt, s);
  if (e == cudaSuccess) e = stable_sort_pairs(key, val, len, key_bits((unsigned)n), kt, vt, s);
  /* kept pairs, their compacted positions, the column counts */
  if (e == cudaSuccess) e = cudaMemsetAsync(cp, 0, ((size_t)n + 1) * sizeof(int), s);
  if (e == cudaSuccess && len > 0) {
    keep_kernel<<<grid_for(len), kThreads, 0, s>>>(key, val, len, n, dedup ? 1 : 0, keep);
    column_count_kernel<<<grid_for(len), kThreads, 0, s>>>(key, keep, len, cp);
    e = cudaGetLastError();
  }
  cnt = reinterpret_cast<int *>(kt); /* the scratch is free again: positions */
  if (e == cudaSuccess && len > 0)
    e = cudaMemcpyAsync(cnt, keep, (size_t)len * sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && len > 0) e = exclusive_scan(cnt, len, cnt, s);
  if (e == cudaSuccess) e = exclusive_scan(cp, (long long)n + 1, cp, s);
  int nnz = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&nnz, cp + n, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(bad_out, dflag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = tbfs::dev_alloc(&ic, (size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
  if (e == cudaSuccess && len > 0) {
    compact_kernel<<<grid_for(len), kThreads, 0, s>>>(val, keep, cnt, len, ic);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  tbfs::dev_free(buf);
  tbfs::dev_free(keep);
  tbfs::dev_free(dflag);
  if (e != cudaSuccess) {
    tbfs::dev_free(cp);
    tbfs::dev_free(ic);
    return e;
  }
  *cp_out = cp;
  *ic_out = ic;
  *nnz_out = nnz;
  return cudaSuccess;
}

cudaError_t mm_parse_device(const char *text, long long len, long long nz, long long M,
                            long long N, int *src, int *dst, long long *lines_out,
                            long long *bad_out, cudaStream_t s) {
  *lines_out = 0;
  *bad_out = -1;
  const long long tiles = (len + kTextTile - 1) / kTextTile;
  if (tiles + 1 > INT32_MAX) return cudaErrorInvalidValue;
  int *offs = nullptr;
  unsigned long long *bad = nullptr;
  cudaError_t e = tbfs::dev_alloc(&offs, (size_t)(tiles + 1) * sizeof(int));
  if (e == cudaSuccess) e = tbfs::dev_alloc(&bad, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(offs, 0, (size_t)(tiles + 1) * sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0xff, sizeof(unsigned long long), s);
  if (e == cudaSuccess && tiles > 0) {
    mm_count_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(text, len, offs);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = exclusive_scan(offs, tiles + 1, offs, s);
  if (e == cudaSuccess && tiles > 0) {
    mm_parse_kernel<<<(unsigned)tiles, kThreads, 0, s>>>(text, len, offs, nz, M, N, src, dst, bad);
    e = cudaGetLastError();
  }
  int lines = 0;
  unsigned long long b = ~0ull;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&lines, offs + tiles, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&b, bad, sizeof(b), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  tbfs::dev_free(offs);
  tbfs::dev_free(bad);
  if (e != cudaSuccess) return e;
  *lines_out = lines;
  *bad_out = b == ~0ull ? -1 : (long long)b;
  return cudaSuccess;
}

}  // namespace tbfs
