/*
 * host_graph.c -- host-side graph construction (no GPU): Matrix Market
 * reader, CSC builder, seeded generators, largest component, root picking.
 *
 * PRNG: xoshiro256** seeded through splitmix64 (Blackman & Vigna, "Scrambled
 * linear pseudorandom number generators", 2018).  Parallel generation draws
 * each fixed-size chunk of work from its own stream seeded by the chunk
 * index, so results do not depend on the number of threads.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "tbfs_graphgen.h"

void tbfs_set_error(const char *fmt, ...);

/* ------------------------------------------------------------------ PRNG */

static uint64_t splitmix64(uint64_t *x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

typedef struct { uint64_t s[4]; } rng_t;

static void rng_seed(rng_t *r, uint64_t seed, uint64_t stream) {
  uint64_t x = seed ^ (stream * 0xd1342543de82ef95ull + 0x2545f4914f6cdd1dull);
  for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(rng_t *r) {
  uint64_t *s = r->s;
  const uint64_t result = rotl64(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return result;
}

/* uniform double in [0,1) with 53 random bits */
static inline double rng_unit(rng_t *r) { return (double)(rng_next(r) >> 11) * 0x1.0p-53; }

/* uniform integer in [0, bound) by 128-bit multiply-high */
static inline uint64_t rng_below(rng_t *r, uint64_t bound) {
  return (uint64_t)(((__uint128_t)rng_next(r) * bound) >> 64);
}

/* ------------------------------------------------------------ threading */

static int num_threads(void) {
  long p = sysconf(_SC_NPROCESSORS_ONLN);
  const char *env = getenv("TBFS_HOST_THREADS");
  if (env && atoi(env) > 0) p = atoi(env);
  if (p < 1) p = 1;
  if (p > 64) p = 64;
  return (int)p;
}

typedef void (*range_fn)(void *ctx, int64_t begin, int64_t end);
typedef struct { range_fn fn; void *ctx; int64_t begin, end; } range_job;

static void *range_thunk(void *arg) {
  range_job *j = (range_job *)arg;
  j->fn(j->ctx, j->begin, j->end);
  return NULL;
}

/* Runs fn over [0,total) split into contiguous ranges, one per thread. */
static void parallel_for(int64_t total, range_fn fn, void *ctx) {
  int t = num_threads();
  if (total < 4096 || t == 1) {
    fn(ctx, 0, total);
    return;
  }
  if (t > total) t = (int)total;
  pthread_t th[64];
  range_job jobs[64];
  int64_t step = (total + t - 1) / t;
  int started = 0;
  for (int i = 0; i < t; ++i) {
    jobs[i].fn = fn;
    jobs[i].ctx = ctx;
    jobs[i].begin = i * step;
    jobs[i].end = (i + 1) * step < total ? (i + 1) * step : total;
    if (jobs[i].begin >= jobs[i].end) continue;
    if (pthread_create(&th[i], NULL, range_thunk, &jobs[i]) != 0) {
      range_thunk(&jobs[i]); /* run inline if a thread cannot start */
      jobs[i].begin = jobs[i].end;
    }
    ++started;
  }
  for (int i = 0; i < t; ++i)
    if (jobs[i].begin < jobs[i].end) pthread_join(th[i], NULL);
  (void)started;
}

/* --------------------------------------------------------- CSC builder */

void tbfs_host_csc_free(tbfs_host_csc *g) {
  if (!g) return;
  free(g->col_ptr);
  free(g->row_idx);
  free(g);
}

static int cmp_i32(const void *a, const void *b) {
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

static void sort_i32(int32_t *a, int64_t len) {
  if (len <= 32) {
    for (int64_t i = 1; i < len; ++i) {
      int32_t v = a[i];
      int64_t j = i - 1;
      while (j >= 0 && a[j] > v) {
        a[j + 1] = a[j];
        --j;
      }
      a[j + 1] = v;
    }
  } else {
    qsort(a, (size_t)len, sizeof(int32_t), cmp_i32);
  }
}

typedef struct {
  int64_t *ptr;     /* column starts before compaction, n+1 */
  int32_t *rows;
  int64_t *newdeg;  /* degree after sort/dedup */
  int dedup;
} colsort_ctx;

static void colsort_range(void *vctx, int64_t b, int64_t e) {
  colsort_ctx *c = (colsort_ctx *)vctx;
  for (int64_t v = b; v < e; ++v) {
    int32_t *a = c->rows + c->ptr[v];
    int64_t len = c->ptr[v + 1] - c->ptr[v];
    sort_i32(a, len);
    if (c->dedup && len > 1) {
      int64_t w = 1;
      for (int64_t i = 1; i < len; ++i)
        if (a[i] != a[w - 1]) a[w++] = a[i];
      len = w;
    }
    c->newdeg[v] = len;
  }
}

tbfs_status tbfs_csc_from_edges(int32_t n, const int32_t *src, const int32_t *dst,
                                int64_t m, uint32_t flags, tbfs_host_csc **out) {
  if (!out || n < 0 || m < 0 || (m > 0 && (!src || !dst))) {
    tbfs_set_error("tbfs_csc_from_edges: invalid arguments");
    return TBFS_ERR_INVALID_ARG;
  }
  *out = NULL;
  const int sym = (flags & TBFS_BUILD_SYMMETRIZE) != 0;
  const int noloop = (flags & TBFS_BUILD_DROP_LOOPS) != 0;
  int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cnt) return TBFS_ERR_OUT_OF_MEMORY;
  for (int64_t k = 0; k < m; ++k) {
    int32_t u = src[k], v = dst[k];
    if (u < 0 || u >= n || v < 0 || v >= n) {
      free(cnt);
      tbfs_set_error("tbfs_csc_from_edges: edge %lld (%d,%d) out of range n=%d",
                     (long long)k, u, v, n);
      return TBFS_ERR_INVALID_ARG;
    }
    if (noloop && u == v) continue;
    cnt[v + 1]++;
    if (sym) cnt[u + 1]++;
  }
  for (int64_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  const int64_t total = cnt[n];
  int32_t *rows = (int32_t *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int32_t));
  int64_t *fill = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
  if (!rows || !fill) {
    free(cnt);
    free(rows);
    free(fill);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  memcpy(fill, cnt, ((size_t)n + 1) * sizeof(int64_t));
  for (int64_t k = 0; k < m; ++k) {
    int32_t u = src[k], v = dst[k];
    if (noloop && u == v) continue;
    rows[fill[v]++] = u;
    if (sym) rows[fill[u]++] = v;
  }
  free(fill);
  int64_t nnz = total;
  if (flags & (TBFS_BUILD_DEDUP | TBFS_BUILD_SORT)) {
    int64_t *newdeg = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    if (!newdeg) {
      free(cnt);
      free(rows);
      return TBFS_ERR_OUT_OF_MEMORY;
    }
    colsort_ctx c = {cnt, rows, newdeg, (flags & TBFS_BUILD_DEDUP) != 0};
    parallel_for(n, colsort_range, &c);
    /* compact forward: new starts never exceed old starts */
    int64_t w = 0;
    for (int64_t v = 0; v < n; ++v) {
      int64_t b = cnt[v], len = newdeg[v];
      if (w != b) memmove(rows + w, rows + b, (size_t)len * sizeof(int32_t));
      cnt[v] = w;
      w += len;
    }
    cnt[n] = w;
    nnz = w;
    free(newdeg);
  }
  if (nnz > INT32_MAX) {
    free(cnt);
    free(rows);
    tbfs_set_error("tbfs_csc_from_edges: nnz %lld exceeds int32 CSC", (long long)nnz);
    return TBFS_ERR_UNSUPPORTED;
  }
  tbfs_host_csc *g = (tbfs_host_csc *)calloc(1, sizeof(*g));
  int32_t *cp = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
  if (!g || !cp) {
    free(g);
    free(cp);
    free(cnt);
    free(rows);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  for (int64_t v = 0; v <= n; ++v) cp[v] = (int32_t)cnt[v];
  free(cnt);
  int32_t *shrunk = (int32_t *)realloc(rows, (size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
  g->n = n;
  g->nnz = nnz;
  g->col_ptr = cp;
  g->row_idx = shrunk ? shrunk : rows;
  *out = g;
  return TBFS_OK;
}

/* ------------------------------------------------------ Matrix Market */

tbfs_status tbfs_mm_read(const char *path, int32_t undirected, tbfs_host_csc **out) {
  if (!path || !out) return TBFS_ERR_INVALID_ARG;
  *out = NULL;
  FILE *f = fopen(path, "r");
  if (!f) {
    tbfs_set_error("tbfs_mm_read: cannot open %s: %s", path, strerror(errno));
    return TBFS_ERR_IO;
  }
  char line[1024];
  if (!fgets(line, sizeof line, f) || strncmp(line, "%%MatrixMarket", 14) != 0) {
    fclose(f);
    tbfs_set_error("tbfs_mm_read: %s has no Matrix Market banner", path);
    return TBFS_ERR_IO;
  }
  if (!strstr(line, "coordinate")) {
    fclose(f);
    tbfs_set_error("tbfs_mm_read: %s is not a coordinate (sparse) file", path);
    return TBFS_ERR_IO;
  }
  long long M = -1, N = -1, nz = -1;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '%') continue;
    if (sscanf(line, "%lld %lld %lld", &M, &N, &nz) == 3) break;
  }
  if (M < 0 || N < 0 || nz < 0 || N > INT32_MAX || M > INT32_MAX) {
    fclose(f);
    tbfs_set_error("tbfs_mm_read: bad size line in %s", path);
    return TBFS_ERR_IO;
  }
  int32_t n = (int32_t)N;
  int32_t *src = (int32_t *)malloc((size_t)(nz > 0 ? nz : 1) * sizeof(int32_t));
  int32_t *dst = (int32_t *)malloc((size_t)(nz > 0 ? nz : 1) * sizeof(int32_t));
  if (!src || !dst) {
    fclose(f);
    free(src);
    free(dst);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  long long k = 0;
  while (k < nz && fgets(line, sizeof line, f)) {
    if (line[0] == '%' || line[0] == '\n') continue;
    long long i, j;
    if (sscanf(line, "%lld %lld", &i, &j) != 2 || i < 1 || j < 1 || i > M || j > N ||
        i > N) {
      fclose(f);
      free(src);
      free(dst);
      tbfs_set_error("tbfs_mm_read: bad entry line %lld in %s", k, path);
      return TBFS_ERR_IO;
    }
    src[k] = (int32_t)(i - 1); /* row i: source of the edge */
    dst[k] = (int32_t)(j - 1); /* column j: target */
    ++k;
  }
  fclose(f);
  if (k != nz) {
    free(src);
    free(dst);
    tbfs_set_error("tbfs_mm_read: %s ends after %lld of %lld entries", path, k, nz);
    return TBFS_ERR_IO;
  }
  /* Undirected: the lower triangle plus its transpose, diagonal kept twice
   * (TurboBFS_CSC_TD/sparseformatransf.c:60-104).  Directed: file order. */
  tbfs_status st = tbfs_csc_from_edges(n, src, dst, nz,
                                       undirected ? TBFS_BUILD_SYMMETRIZE : 0u, out);
  free(src);
  free(dst);
  return st;
}

/* ---------------------------------------------------------- generators */

static uint64_t edge_key(int32_t u, int32_t v) {
  uint32_t a = (uint32_t)(u < v ? u : v), b = (uint32_t)(u < v ? v : u);
  return ((uint64_t)a << 32) | b;
}

typedef struct {
  uint64_t *slots;
  uint64_t mask;
} hset;

static int hset_init(hset *h, int64_t expect) {
  uint64_t cap = 1024;
  while (cap < (uint64_t)expect * 2) cap <<= 1;
  h->slots = (uint64_t *)malloc(cap * sizeof(uint64_t));
  if (!h->slots) return 0;
  memset(h->slots, 0xff, cap * sizeof(uint64_t));
  h->mask = cap - 1;
  return 1;
}

/* returns 1 if inserted, 0 if already present */
static int hset_insert(hset *h, uint64_t key) {
  uint64_t x = key;
  uint64_t i = splitmix64(&x) & h->mask;
  while (h->slots[i] != UINT64_MAX) {
    if (h->slots[i] == key) return 0;
    i = (i + 1) & h->mask;
  }
  h->slots[i] = key;
  return 1;
}

tbfs_status tbfs_gen_er(int32_t n, int64_t m, uint64_t seed, tbfs_host_csc **out) {
  if (!out || n < 2 || m < 0 || (double)m > 0.5 * (double)n * (double)(n - 1)) {
    tbfs_set_error("tbfs_gen_er: invalid n=%d m=%lld", n, (long long)m);
    return TBFS_ERR_INVALID_ARG;
  }
  int32_t *src = (int32_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
  int32_t *dst = (int32_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
  hset h;
  if (!src || !dst || !hset_init(&h, m)) {
    free(src);
    free(dst);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  rng_t r;
  rng_seed(&r, seed, 0);
  int64_t k = 0;
  while (k < m) {
    int32_t u = (int32_t)rng_below(&r, (uint64_t)n);
    int32_t v = (int32_t)rng_below(&r, (uint64_t)n);
    if (u == v) continue;
    if (!hset_insert(&h, edge_key(u, v))) continue;
    src[k] = u;
    dst[k] = v;
    ++k;
  }
  free(h.slots);
  tbfs_status st = tbfs_csc_from_edges(
      n, src, dst, m, TBFS_BUILD_SYMMETRIZE | TBFS_BUILD_DROP_LOOPS | TBFS_BUILD_DEDUP, out);
  free(src);
  free(dst);
  return st;
}

#define RMAT_CHUNK (1 << 20)

typedef struct {
  int32_t scale;
  double a, ab, abc;
  uint64_t seed;
  int64_t m;
  int32_t *src, *dst;
  const int32_t *perm;
} rmat_ctx;

static void rmat_range(void *vctx, int64_t cb, int64_t ce) {
  rmat_ctx *c = (rmat_ctx *)vctx;
  for (int64_t chunk = cb; chunk < ce; ++chunk) {
    rng_t r;
    rng_seed(&r, c->seed, (uint64_t)chunk + 1);
    int64_t e0 = chunk * (int64_t)RMAT_CHUNK;
    int64_t e1 = e0 + RMAT_CHUNK < c->m ? e0 + RMAT_CHUNK : c->m;
    for (int64_t e = e0; e < e1; ++e) {
      uint32_t u = 0, v = 0;
      for (int b = 0; b < c->scale; ++b) {
        double x = rng_unit(&r);
        uint32_t ub = 0, vb = 0;
        if (x < c->a) {
        } else if (x < c->ab) {
          vb = 1;
        } else if (x < c->abc) {
          ub = 1;
        } else {
          ub = 1;
          vb = 1;
        }
        u = (u << 1) | ub;
        v = (v << 1) | vb;
      }
      c->src[e] = (int32_t)u;
      c->dst[e] = (int32_t)v;
    }
  }
}

typedef struct {
  int32_t *src, *dst;
  const int32_t *perm;
} relabel_ctx;

static void relabel_range(void *vctx, int64_t b, int64_t e) {
  relabel_ctx *c = (relabel_ctx *)vctx;
  for (int64_t k = b; k < e; ++k) {
    c->src[k] = c->perm[c->src[k]];
    c->dst[k] = c->perm[c->dst[k]];
  }
}

tbfs_status tbfs_gen_rmat(int32_t scale, int32_t edgefactor, double a, double b,
                          double c, uint64_t seed, int32_t permute,
                          tbfs_host_csc **out) {
  if (!out || scale < 1 || scale > 30 || edgefactor < 1 || a < 0 || b < 0 || c < 0 ||
      a + b + c > 1.0) {
    tbfs_set_error("tbfs_gen_rmat: invalid arguments");
    return TBFS_ERR_INVALID_ARG;
  }
  const int32_t n = (int32_t)1 << scale;
  const int64_t m = (int64_t)edgefactor << scale;
  rmat_ctx ctx;
  ctx.scale = scale;
  ctx.a = a;
  ctx.ab = a + b;
  ctx.abc = a + b + c;
  ctx.seed = seed;
  ctx.m = m;
  ctx.src = (int32_t *)malloc((size_t)m * sizeof(int32_t));
  ctx.dst = (int32_t *)malloc((size_t)m * sizeof(int32_t));
  ctx.perm = NULL;
  if (!ctx.src || !ctx.dst) {
    free(ctx.src);
    free(ctx.dst);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  int64_t chunks = (m + RMAT_CHUNK - 1) / RMAT_CHUNK;
  int t = num_threads();
  if (chunks < 2 || t == 1) {
    rmat_range(&ctx, 0, chunks);
  } else {
    /* parallel over chunks: thread i takes a contiguous chunk range */
    pthread_t th[64];
    range_job jobs[64];
    if (t > chunks) t = (int)chunks;
    int64_t step = (chunks + t - 1) / t;
    for (int i = 0; i < t; ++i) {
      jobs[i].fn = rmat_range;
      jobs[i].ctx = &ctx;
      jobs[i].begin = i * step;
      jobs[i].end = (i + 1) * step < chunks ? (i + 1) * step : chunks;
      if (jobs[i].begin >= jobs[i].end) continue;
      if (pthread_create(&th[i], NULL, range_thunk, &jobs[i]) != 0) {
        range_thunk(&jobs[i]);
        jobs[i].begin = jobs[i].end;
      }
    }
    for (int i = 0; i < t; ++i)
      if (jobs[i].begin < jobs[i].end) pthread_join(th[i], NULL);
  }
  if (permute) {
    int32_t *perm = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!perm) {
      free(ctx.src);
      free(ctx.dst);
      return TBFS_ERR_OUT_OF_MEMORY;
    }
    for (int32_t i = 0; i < n; ++i) perm[i] = i;
    rng_t r;
    rng_seed(&r, seed, 0);
    for (int64_t i = n - 1; i > 0; --i) { /* Fisher-Yates */
      int64_t j = (int64_t)rng_below(&r, (uint64_t)i + 1);
      int32_t tmp = perm[i];
      perm[i] = perm[j];
      perm[j] = tmp;
    }
    relabel_ctx rc = {ctx.src, ctx.dst, perm};
    parallel_for(m, relabel_range, &rc);
    free(perm);
  }
  tbfs_status st = tbfs_csc_from_edges(
      n, ctx.src, ctx.dst, m,
      TBFS_BUILD_SYMMETRIZE | TBFS_BUILD_DROP_LOOPS | TBFS_BUILD_DEDUP, out);
  free(ctx.src);
  free(ctx.dst);
  return st;
}

tbfs_status tbfs_gen_grid(int32_t side, double delete_frac, double chord_frac,
                          int32_t max_dist, int32_t max_deg, uint64_t seed,
                          tbfs_host_csc **out) {
  if (!out || side < 2 || (int64_t)side * side > INT32_MAX || delete_frac < 0 ||
      delete_frac >= 1 || chord_frac < 0 || max_dist < 2 || max_deg < 1) {
    tbfs_set_error("tbfs_gen_grid: invalid arguments");
    return TBFS_ERR_INVALID_ARG;
  }
  const int64_t n = (int64_t)side * side;
  const int64_t E = 2 * (int64_t)side * (side - 1);
  /* grid edge e: e < side*(side-1) horizontal (x,y)-(x+1,y), else vertical */
  const int64_t nh = (int64_t)side * (side - 1);
  int64_t ndel = (int64_t)(delete_frac * (double)E + 0.5);
  int32_t *idx = (int32_t *)malloc((size_t)E * sizeof(int32_t));
  uint8_t *deg = (uint8_t *)calloc((size_t)n, 1);
  if (!idx || !deg) {
    free(idx);
    free(deg);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  for (int64_t e = 0; e < E; ++e) idx[e] = (int32_t)e;
  rng_t r;
  rng_seed(&r, seed, 0);
  for (int64_t i = 0; i < ndel; ++i) { /* partial Fisher-Yates: first ndel deleted */
    int64_t j = i + (int64_t)rng_below(&r, (uint64_t)(E - i));
    int32_t t = idx[i];
    idx[i] = idx[j];
    idx[j] = t;
  }
  const int64_t kept = E - ndel;
  const int64_t nchord = (int64_t)(chord_frac * (double)kept + 0.5);
  int32_t *src = (int32_t *)malloc((size_t)(kept + nchord) * sizeof(int32_t));
  int32_t *dst = (int32_t *)malloc((size_t)(kept + nchord) * sizeof(int32_t));
  if (!src || !dst) {
    free(idx);
    free(deg);
    free(src);
    free(dst);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  int64_t m = 0;
  for (int64_t i = ndel; i < E; ++i) {
    int64_t e = idx[i];
    int64_t u, v;
    if (e < nh) {
      int64_t y = e / (side - 1), x = e % (side - 1);
      u = y * side + x;
      v = u + 1;
    } else {
      int64_t f = e - nh;
      int64_t y = f / side, x = f % side;
      u = y * side + x;
      v = u + side;
    }
    src[m] = (int32_t)u;
    dst[m] = (int32_t)v;
    deg[u]++;
    deg[v]++;
    ++m;
  }
  free(idx);
  /* offsets with 2 <= |dx|+|dy| <= max_dist */
  int32_t noff = 0;
  int32_t *offx = (int32_t *)malloc((size_t)(4 * max_dist + 1) * (4 * max_dist + 1) * sizeof(int32_t));
  int32_t *offy = (int32_t *)malloc((size_t)(4 * max_dist + 1) * (4 * max_dist + 1) * sizeof(int32_t));
  hset h;
  if (!offx || !offy || !hset_init(&h, nchord + 16)) {
    free(offx);
    free(offy);
    free(deg);
    free(src);
    free(dst);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  for (int32_t dy = -max_dist; dy <= max_dist; ++dy)
    for (int32_t dx = -max_dist; dx <= max_dist; ++dx) {
      int32_t dd = (dx < 0 ? -dx : dx) + (dy < 0 ? -dy : dy);
      if (dd >= 2 && dd <= max_dist) {
        offx[noff] = dx;
        offy[noff] = dy;
        ++noff;
      }
    }
  int64_t added = 0, attempts = 0, max_attempts = 200 * nchord + 1000;
  while (added < nchord && attempts < max_attempts) {
    ++attempts;
    int64_t u = (int64_t)rng_below(&r, (uint64_t)n);
    int32_t o = (int32_t)rng_below(&r, (uint64_t)noff);
    int64_t ux = u % side, uy = u / side;
    int64_t vx = ux + offx[o], vy = uy + offy[o];
    if (vx < 0 || vy < 0 || vx >= side || vy >= side) continue;
    int64_t v = vy * side + vx;
    if (deg[u] >= max_deg || deg[v] >= max_deg) continue;
    if (!hset_insert(&h, edge_key((int32_t)u, (int32_t)v))) continue;
    src[m] = (int32_t)u;
    dst[m] = (int32_t)v;
    deg[u]++;
    deg[v]++;
    ++m;
    ++added;
  }
  free(h.slots);
  free(offx);
  free(offy);
  free(deg);
  tbfs_status st = tbfs_csc_from_edges((int32_t)n, src, dst, m,
                                       TBFS_BUILD_SYMMETRIZE | TBFS_BUILD_DROP_LOOPS |
                                           TBFS_BUILD_DEDUP,
                                       out);
  free(src);
  free(dst);
  return st;
}

/* ---------------------------------------------------- components, roots */

static int32_t uf_find(int32_t *p, int32_t x) {
  while (p[x] != x) {
    p[x] = p[p[x]];
    x = p[x];
  }
  return x;
}

tbfs_status tbfs_largest_component(const tbfs_host_csc *g, uint8_t *in_lcc,
                                   int64_t *lcc_size) {
  if (!g || !in_lcc) return TBFS_ERR_INVALID_ARG;
  const int32_t n = g->n;
  int32_t *p = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  int64_t *sz = (int64_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t));
  if (!p || !sz) {
    free(p);
    free(sz);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  for (int32_t v = 0; v < n; ++v) p[v] = v;
  for (int32_t v = 0; v < n; ++v)
    for (int64_t k = g->col_ptr[v]; k < g->col_ptr[v + 1]; ++k) {
      int32_t a = uf_find(p, g->row_idx[k]), b = uf_find(p, v);
      if (a != b) {
        if (a < b) p[b] = a;
        else p[a] = b;
      }
    }
  int32_t best = 0;
  for (int32_t v = 0; v < n; ++v) {
    int32_t root = uf_find(p, v);
    if (++sz[root] > sz[best] || (sz[root] == sz[best] && root < best)) best = root;
  }
  int64_t cnt = 0;
  for (int32_t v = 0; v < n; ++v) {
    in_lcc[v] = (uint8_t)(uf_find(p, v) == best);
    cnt += in_lcc[v];
  }
  if (lcc_size) *lcc_size = cnt;
  free(p);
  free(sz);
  return TBFS_OK;
}

tbfs_status tbfs_pick_roots(const tbfs_host_csc *g, int32_t k, uint64_t seed,
                            int32_t *roots) {
  if (!g || !roots || k < 0) return TBFS_ERR_INVALID_ARG;
  uint8_t *in = (uint8_t *)malloc((size_t)(g->n > 0 ? g->n : 1));
  if (!in) return TBFS_ERR_OUT_OF_MEMORY;
  int64_t cnt = 0;
  tbfs_status st = tbfs_largest_component(g, in, &cnt);
  if (st != TBFS_OK) {
    free(in);
    return st;
  }
  if (cnt < k) {
    free(in);
    tbfs_set_error("tbfs_pick_roots: component has %lld < %d vertices", (long long)cnt, k);
    return TBFS_ERR_INVALID_ARG;
  }
  int32_t *ids = (int32_t *)malloc((size_t)(cnt > 0 ? cnt : 1) * sizeof(int32_t));
  if (!ids) {
    free(in);
    return TBFS_ERR_OUT_OF_MEMORY;
  }
  int64_t w = 0;
  for (int32_t v = 0; v < g->n; ++v)
    if (in[v]) ids[w++] = v;
  rng_t r;
  rng_seed(&r, seed, 0x726f6f74ull);
  for (int32_t i = 0; i < k; ++i) {
    int64_t j = i + (int64_t)rng_below(&r, (uint64_t)(cnt - i));
    int32_t t = ids[i];
    ids[i] = ids[j];
    ids[j] = t;
    roots[i] = ids[i];
  }
  free(ids);
  free(in);
  return TBFS_OK;
}

tbfs_status tbfs_degree_profile(const tbfs_host_csc *g, int64_t *hist40,
                                int64_t *max_degree, double *mean_degree) {
  if (!g || !hist40) return TBFS_ERR_INVALID_ARG;
  memset(hist40, 0, 40 * sizeof(int64_t));
  int64_t mx = 0;
  for (int32_t v = 0; v < g->n; ++v) {
    int64_t d = (int64_t)g->col_ptr[v + 1] - g->col_ptr[v];
    if (d > mx) mx = d;
    int b = 0;
    uint64_t x = (uint64_t)d + 1;
    while (x > 1) {
      x >>= 1;
      ++b;
    }
    hist40[b < 40 ? b : 39]++;
  }
  if (max_degree) *max_degree = mx;
  if (mean_degree) *mean_degree = g->n > 0 ? (double)g->nnz / g->n : 0.0;
  return TBFS_OK;
}
