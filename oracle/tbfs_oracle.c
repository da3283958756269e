/*
 * tbfs_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of the
 * reference TurboBFS BFS variants and of what its GPU drivers return.  Used
 * as the parity checker and as the timed CPU baseline; never part of the
 * product path.  Citations are to files of the reference project.
 *
 * Arithmetic notes kept identical to the reference:
 *  - float sums are accumulated in column order, in single precision, and
 *    compared against the double constants 0.1 / 0.9 / 0.01 as the
 *    reference's C does;
 *  - int32 sums wrap in two's complement (done here in uint32 arithmetic so
 *    the wrap is defined behaviour).
 */
#define _GNU_SOURCE
#include "tbfs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static inline int32_t wrap_add(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}

/* ---------------------------------------------- sequential CSC, float sigma */

/* TurboBFS_CSC_TD/bfstdcsc_seq.c:27-96 with the helpers of
 * bfstdcsc_seq_utils.c:21-103 and the SpMV of spmvcsc_seq.c:22-41. */
int oracle_seq_csc_f32(const int *IC, const int *CP, int *S, float *sigma, int r,
                       int nz, int n, int init_S) {
  (void)nz;
  float *f = (float *)calloc((size_t)n + 1, sizeof(float));
  float *ft = (float *)calloc((size_t)n + 1, sizeof(float));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  f[r] = 1.0f;
  if (init_S) {
    for (int i = 0; i < n; ++i) S[i] = -1;
    S[r] = 0;
  }
  int d = 0, c = 1;
  while (c > 0) {
    d++;
    for (int k = 0; k < n; ++k) /* sigma += f   (sum_vs) */
      if (f[k] > 0.1) sigma[k] += f[k];
    for (int i = 0; i < n; ++i) { /* f_t = A^T f over every column (spmv) */
      float sum = 0.0f;
      for (int k = CP[i]; k < CP[i + 1]; ++k) sum += f[IC[k]];
      ft[i] = (sum > 0.1) ? sum : 0.0f;
    }
    for (int k = 0; k < n; ++k) f[k] = (ft[k] > 0.1) ? ft[k] : 0.0f; /* assign_v */
    for (int k = 0; k < n; ++k)                                      /* mult_vs */
      if (sigma[k] > 0.1) f[k] = 0.0f;
    for (int k = 0; k < n; ++k) /* S_v */
      if (f[k] > 0.9) S[k] = d;
    c = 0; /* check_f */
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.9) {
        c = 1;
        break;
      }
  }
  free(f);
  free(ft);
  return d;
}

/* ---------------------------------------------- sequential CSC, int sigma */

/* TurboBFS_CSC_TDBU/bfstdcsc_seq.c:26-96: the same level loop in int32. */
int oracle_seq_csc_i32(const int *IC, const int *CP, int *S, int *sigma, int r,
                       int nz, int n) {
  (void)nz;
  int32_t *f = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  int32_t *ft = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  f[r] = 1;
  for (int i = 0; i < n; ++i) S[i] = -1;
  S[r] = 0;
  int d = 0, c = 1;
  while (c > 0) {
    d++;
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.1) sigma[k] = wrap_add(sigma[k], f[k]);
    for (int i = 0; i < n; ++i) {
      int32_t sum = 0;
      for (int k = CP[i]; k < CP[i + 1]; ++k) sum = wrap_add(sum, f[IC[k]]);
      ft[i] = (sum > 0.1) ? sum : 0;
    }
    for (int k = 0; k < n; ++k) f[k] = (ft[k] > 0.1) ? ft[k] : 0;
    for (int k = 0; k < n; ++k)
      if (sigma[k] > 0.1) f[k] = 0;
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.9) S[k] = d;
    c = 0;
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.9) {
        c = 1;
        break;
      }
  }
  free(f);
  free(ft);
  return d;
}

/* --------------------------------------------------- sequential COOC */

/* TurboBFS_COOC_TD/bfstdcooc_seq.c:29-91 with spmvcooc_seq.c:27-36: f_t is
 * accumulated across levels and never cleared. */
int oracle_seq_cooc_f32(const int *I, const int *J, float *sigma, int r, int nz,
                        int n) {
  float *f = (float *)calloc((size_t)n + 1, sizeof(float));
  float *ft = (float *)calloc((size_t)n + 1, sizeof(float));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  f[r] = 1.0f;
  int d = 0, c = 1;
  while (c > 0) {
    d++;
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.1) sigma[k] += f[k];
    for (int i = 0; i < nz; ++i) ft[J[i]] += f[I[i]];
    for (int k = 0; k < n; ++k) f[k] = (ft[k] > 0.1) ? ft[k] : 0.0f;
    for (int k = 0; k < n; ++k)
      if (sigma[k] > 0.1) f[k] = 0.0f;
    c = 0;
    for (int k = 0; k < n; ++k)
      if (f[k] > 0.9) {
        c = 1;
        break;
      }
  }
  free(f);
  free(ft);
  return d;
}

/* ------------------------------------------------------------ exact BFS */

typedef unsigned __int128 u128;
static const u128 SAT = ((u128)1) << 100; /* saturation ceiling, >> 2^63 */

static inline u128 sat_add(u128 a, u128 b) {
  u128 s = a + b;
  return s > SAT ? SAT : s;
}

/* Level-synchronous BFS: discovery by push over out-lists (the transpose of
 * the CSC, built here), then sigma[v] = sum of sigma[u] over in-list entries
 * u of v with S[u] = S[v]-1: the number of shortest paths counted with the
 * multiplicity of the CSC entries, as in the reference's semiring. */
int oracle_exact_bfs(const int *CP, const int *IC, int n, int r, int *S,
                     int64_t *sigma, uint8_t *ovf) {
  const int64_t nnz = CP[n];
  int64_t *rp = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int32_t *jr = (int32_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
  int32_t *q = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  u128 *sg = (u128 *)calloc((size_t)n + 1, sizeof(u128));
  if (!rp || !jr || !q || !sg) {
    free(rp);
    free(jr);
    free(q);
    free(sg);
    return -1;
  }
  for (int64_t k = 0; k < nnz; ++k) rp[IC[k] + 1]++;
  for (int v = 0; v < n; ++v) rp[v + 1] += rp[v];
  {
    int64_t *fill = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    if (!fill) {
      free(rp);
      free(jr);
      free(q);
      free(sg);
      return -1;
    }
    memcpy(fill, rp, ((size_t)n + 1) * sizeof(int64_t));
    for (int v = 0; v < n; ++v)
      for (int64_t k = CP[v]; k < CP[v + 1]; ++k) jr[fill[IC[k]]++] = v;
    free(fill);
  }
  for (int v = 0; v < n; ++v) S[v] = -1;
  S[r] = 0;
  sg[r] = 1;
  int64_t head = 0, tail = 0;
  q[tail++] = r;
  int levels = 0;
  while (head < tail) {
    int64_t lvl_end = tail;
    ++levels;
    int d = S[q[head]];
    for (int64_t i = head; i < lvl_end; ++i) {
      int u = q[i];
      for (int64_t k = rp[u]; k < rp[u + 1]; ++k) {
        int v = jr[k];
        if (S[v] == -1) {
          S[v] = d + 1;
          q[tail++] = v;
        }
      }
    }
    for (int64_t i = lvl_end; i < tail; ++i) {
      int v = q[i];
      u128 s = 0;
      for (int64_t k = CP[v]; k < CP[v + 1]; ++k)
        if (S[IC[k]] == d) s = sat_add(s, sg[IC[k]]);
      sg[v] = s;
    }
    head = lvl_end;
  }
  const u128 LIM = ((u128)1) << 63;
  for (int v = 0; v < n; ++v) {
    if (sg[v] >= LIM) {
      ovf[v] = 1;
      sigma[v] = -1;
    } else {
      ovf[v] = 0;
      sigma[v] = (int64_t)sg[v];
    }
  }
  free(rp);
  free(jr);
  free(q);
  free(sg);
  return levels;
}

/* ---------------------------------------------- reference GPU emulations */

/* bfsgputdcsc_sc.cu:95-119 driving spMvUgCscScKernel (:159-185) and
 * bfsFunctionsKernel (:194-208).  The warp variant (bfsgputdcsc_wa.cu) writes
 * ft for every unvisited column after a memset, which leaves the same ft. */
int oracle_gpu_td_csc(const int *IC, const int *CP, int *S, float *sigma, int r,
                      int nz, int n) {
  (void)nz;
  int32_t *f = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  int32_t *ft = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  for (int i = 0; i < n; ++i) {
    S[i] = 0;
    sigma[i] = 0.0f;
  }
  int d = 0, c = 1;
  while (c) {
    d++;
    c = 0;
    if (d == 1) {
      f[r] = 1;
      sigma[r] = 1.0f;
    }
    for (int i = 0; i < n; ++i) {
      ft[i] = 0;
      if (sigma[i] < 0.01) {
        int32_t sum = 0;
        for (int k = CP[i]; k < CP[i + 1]; ++k) sum = wrap_add(sum, f[IC[k]]);
        if (sum > 0.9) ft[i] = sum;
      }
    }
    for (int i = 0; i < n; ++i) {
      f[i] = 0;
      if (ft[i] > 0.9) {
        c = 1;
        f[i] = ft[i];
        sigma[i] += (float)ft[i];
        S[i] = d;
      }
    }
  }
  free(f);
  free(ft);
  return d;
}

/* bfsgpubucsc_sc.cu:79-95 driving bfsBuScKernel (:122-148).  Writes of d+1
 * during a level never equal the tested value d, so the kernel's result is
 * the sequential one below. */
int oracle_gpu_bu_csc(const int *IC, const int *CP, int *S, int r, int nz, int n) {
  (void)nz;
  for (int i = 0; i < n; ++i) S[i] = -1;
  int d = 0, c = 1;
  while (c) {
    c = 0;
    if (d == 0) S[r] = 0;
    for (int i = 0; i < n; ++i) {
      if (S[i] != -1) continue;
      for (int k = CP[i]; k < CP[i + 1]; ++k)
        if (S[IC[k]] == d) {
          S[i] = d + 1;
          c = 1;
          break;
        }
    }
    d++;
  }
  return d;
}

/* bfsgputdbucsc_sc.cu:106-153: top-down levels (BfsCscScKernel :199-229 and
 * fKernel :235-246) while the float counter sizef of the last top-down level
 * is <= 0.001f*n, then bottom-up levels (bfsBuScKernel :254-278) to the end.
 * *switch_level receives the depth d of the first bottom-up level (its
 * parents' depth) or -1 if the run stayed top-down. */
int oracle_gpu_tdbu_csc(const int *IC, const int *CP, int *S, int *sigma, int r,
                        int nz, int n, int *switch_level) {
  (void)nz;
  int32_t *f = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  int32_t *ft = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  for (int i = 0; i < n; ++i) {
    S[i] = -1;
    sigma[i] = 0;
  }
  int d = 0, c = 1;
  float sizef = 0.0f;
  float thr_td = 0.001f;
  float thresh_td = thr_td * (float)n;
  if (switch_level) *switch_level = -1;
  while (c) {
    c = 0;
    if (sizef <= thresh_td) {
      sizef = 0.0f;
      d++;
      if (d == 1) {
        f[r] = 1;
        sigma[r] = 1;
        S[r] = 0;
      }
      for (int i = 0; i < n; ++i) {
        ft[i] = 0;
        if (sigma[i] < 0.01) {
          int32_t sum = 0;
          for (int k = CP[i]; k < CP[i + 1]; ++k) sum = wrap_add(sum, f[IC[k]]);
          if (sum > 0.9) {
            ft[i] = sum;
            sigma[i] = wrap_add(sigma[i], ft[i]);
            if (S[i] == -1) S[i] = d;
            c = 1;
          }
        }
      }
      for (int i = 0; i < n; ++i) {
        f[i] = 0;
        if (ft[i] > 0.9) {
          f[i] = ft[i];
          sizef += 1.0f;
        }
      }
    } else {
      if (switch_level && *switch_level < 0) *switch_level = d;
      if (d == 0) S[r] = 0;
      for (int i = 0; i < n; ++i) {
        if (S[i] != -1) continue;
        for (int k = CP[i]; k < CP[i + 1]; ++k)
          if (S[IC[k]] == d) {
            S[i] = d + 1;
            c = 1;
            break;
          }
      }
      d++;
    }
  }
  free(f);
  free(ft);
  return d;
}

/* bfsgputdcooc_sc.cu:89-115 driving spMvUgCoocScKernel (:152-167) and
 * bfsFunctionsKernel (:175-188). */
int oracle_gpu_td_cooc(const int *I, const int *J, float *sigma, int r, int nz,
                       int n) {
  int32_t *f = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  int32_t *ft = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  if (!f || !ft) {
    free(f);
    free(ft);
    return -1;
  }
  for (int i = 0; i < n; ++i) sigma[i] = 0.0f;
  int d = 0, c = 1;
  while (c) {
    d++;
    c = 0;
    memset(ft, 0, (size_t)n * sizeof(int32_t));
    if (d == 1) {
      f[r] = 1;
      sigma[r] = 1.0f;
    }
    for (int i = 0; i < nz; ++i)
      if (f[I[i]] != 0) ft[J[i]] = wrap_add(ft[J[i]], f[I[i]]);
    for (int i = 0; i < n; ++i) {
      f[i] = 0;
      if (sigma[i] < 0.01) f[i] = ft[i];
      if (f[i] > 0) {
        c = 1;
        sigma[i] += (float)f[i];
      }
    }
  }
  free(f);
  free(ft);
  return d;
}

/* ----------------------------------------------------- CPU baseline runner */

typedef struct {
  const int *IC, *CP;
  int nz, n;
  const int *roots;
  int k;
  int next; /* guarded by mu */
  pthread_mutex_t mu;
  double *seconds;
  int64_t *edges;
} many_ctx;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void *many_worker(void *arg) {
  many_ctx *c = (many_ctx *)arg;
  int *S = (int *)malloc((size_t)c->n * sizeof(int));
  int *sg = (int *)malloc((size_t)c->n * sizeof(int));
  if (!S || !sg) {
    free(S);
    free(sg);
    return NULL;
  }
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int i = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (i >= c->k) break;
    memset(sg, 0, (size_t)c->n * sizeof(int));
    double t0 = now_s();
    oracle_seq_csc_i32(c->IC, c->CP, S, sg, c->roots[i], c->nz, c->n);
    double t1 = now_s();
    int64_t e = 0;
    for (int v = 0; v < c->n; ++v)
      if (S[v] >= 0) e += c->CP[v + 1] - c->CP[v];
    if (c->seconds) c->seconds[i] = t1 - t0;
    if (c->edges) c->edges[i] = e;
  }
  free(S);
  free(sg);
  return NULL;
}

double oracle_seq_many(const int *IC, const int *CP, int nz, int n,
                       const int *roots, int k, int threads, double *seconds,
                       int64_t *edges) {
  many_ctx c;
  c.IC = IC;
  c.CP = CP;
  c.nz = nz;
  c.n = n;
  c.roots = roots;
  c.k = k;
  c.next = 0;
  c.seconds = seconds;
  c.edges = edges;
  pthread_mutex_init(&c.mu, NULL);
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  int started = 0;
  double t0 = now_s();
  for (int t = 0; t < threads; ++t)
    if (pthread_create(&th[t], NULL, many_worker, &c) == 0) ++started;
  if (started == 0) many_worker(&c);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  double t1 = now_s();
  pthread_mutex_destroy(&c.mu);
  return t1 - t0;
}


/* ------------------------------------------------------------------
 * Betweenness centrality (not in the reference: the dependency sweep of
 * U. Brandes, J. Math. Sociology 25(2), 2001, on top of the reference's
 * forward quantities S and sigma).  Restates the summation order of the
 * library's GPU sweep so that results can be compared bit for bit:
 * delta[v] = sigma[v] * sum of q[w] = (1 + delta[w]) / sigma[w] over the
 * out-list entries v -> w with S[w] = S[v] + 1 (Brandes' sum with sigma[v]
 * factored out); the sum below 32 entries in list order,
 * otherwise per segment of BRANDES_SEG entries 32 strided partial sums
 * (entries l, l+32, ...) combined by a butterfly (xor 16, 8, 4, 2, 1), the
 * segment sums added in segment order.  Built with -ffp-contract=off so that
 * no multiply-add is fused.  (orp, ojr): out-lists; bc accumulates over
 * the roots in order; returns the number of roots whose counts wrapped.
 * ------------------------------------------------------------------ */
/* segment length of the dependency sums of lists of 32 entries or more */
#define BRANDES_SEG 2048

int oracle_brandes(const int *orp, const int *ojr, int n, const int *roots, int k, double *bc) {
  int *S = (int *)malloc((size_t)n * sizeof(int));
  uint64_t *sg = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
  int *q = (int *)malloc((size_t)n * sizeof(int));
  double *delta = (double *)malloc((size_t)n * sizeof(double));
  int ovf_roots = 0;
  memset(bc, 0, (size_t)n * sizeof(double));
  for (int ri = 0; ri < k; ++ri) {
    const int r = roots[ri];
    for (int v = 0; v < n; ++v) {
      S[v] = -1;
      sg[v] = 0;
      delta[v] = 0.0;
    }
    int head = 0, tail = 0, ovf = 0;
    S[r] = 0;
    sg[r] = 1;
    q[tail++] = r;
    while (head < tail) { /* queue order = depth order */
      const int u = q[head++];
      for (int e = orp[u]; e < orp[u + 1]; ++e) {
        const int w = ojr[e];
        if (S[w] < 0) {
          S[w] = S[u] + 1;
          q[tail++] = w;
        }
        if (S[w] == S[u] + 1) {
          const uint64_t t = sg[w] + sg[u];
          if (t < sg[w] || (t >> 63)) ovf = 1;
          sg[w] = t;
        }
      }
    }
    ovf_roots += ovf;
    for (int i = tail - 1; i >= 0; --i) { /* deepest first */
      const int v = q[i];
      const int d = S[v], b = orp[v], e = orp[v + 1];
      const double sv = (double)sg[v];
      double acc = 0.0; /* sum of the children's q = (1 + delta) / sigma */
      if (e - b < 32) {
        for (int j = b; j < e; ++j) {
          const int w = ojr[j];
          if (S[w] == d + 1) acc = acc + delta[w];
        }
      } else { /* segments of BRANDES_SEG entries, their sums in order */
        for (int sb = b; sb < e; sb += BRANDES_SEG) {
          const int se = sb + BRANDES_SEG < e ? sb + BRANDES_SEG : e;
          double part[32], nxt[32];
          for (int l = 0; l < 32; ++l) {
            double a = 0.0;
            for (int j = sb + l; j < se; j += 32) {
              const int w = ojr[j];
              if (S[w] == d + 1) a = a + delta[w];
            }
            part[l] = a;
          }
          for (int o = 16; o > 0; o >>= 1) {
            for (int l = 0; l < 32; ++l) nxt[l] = part[l] + part[l ^ o];
            memcpy(part, nxt, sizeof(part));
          }
          acc = sb == b ? part[0] : acc + part[0];
        }
      }
      const double dv = sv * acc;
      delta[v] = (1.0 + dv) / sv; /* q[v], what its parents add */
      if (v != r) bc[v] = bc[v] + dv;
    }
  }
  free(S);
  free(sg);
  free(q);
  free(delta);
  return ovf_roots;
}

/* ------------------------------------------------------ degree statistics */

/* degree_max (TurboBFS_CSC_TD/degree.c:36-48): strict '>' keeps the first
 * vertex of the maximum.  degree_sta (:54-76): mean = sum / n; variance =
 * sum of pow(deg - mean, 2) in vertex order / (n - 1).  degree_dist,
 * degree_dist_rel, degree_dist_ac (:83-141): per-degree counts, percentages
 * 100 * count / n, then buckets 0 and 1 copied and every later bucket
 * [low, 2 low) summed in degree order into entry `low` while low < max. */
int oracle_degree_stats(const int *deg, int n, int64_t *maxd, int64_t *argmax, double *mean,
                        double *sd, int64_t *dist_ac, double *dist_rel_ac, int cap) {
  int64_t mx = 0, ix = -1, sum = 0;
  for (int i = 0; i < n; ++i) {
    if (deg[i] > mx) {
      mx = deg[i];
      ix = i;
    }
    sum += deg[i];
  }
  const double m = n ? (double)sum / (double)n : 0.0;
  double ss = 0.0;
  for (int i = 0; i < n; ++i) ss += pow((double)deg[i] - m, 2);
  *maxd = mx;
  *argmax = ix;
  *mean = m;
  *sd = sqrt(ss / (double)(n - 1));
  int need = 2;
  for (int64_t low = 2; low < mx; low *= 2) ++need;
  if (cap < need) return -1;
  int64_t *dist = (int64_t *)calloc((size_t)mx + 1, sizeof(int64_t));
  double *rel = (double *)calloc((size_t)mx + 1, sizeof(double));
  if (!dist || !rel) {
    free(dist);
    free(rel);
    return -1;
  }
  for (int i = 0; i < n; ++i) dist[deg[i]]++;
  for (int64_t d = 0; d <= mx; ++d) rel[d] = (double)dist[d] * 100.0 / ((double)n);
  memset(dist_ac, 0, (size_t)cap * sizeof(int64_t));
  memset(dist_rel_ac, 0, (size_t)cap * sizeof(double));
  for (int b = 0; b < 2 && b <= mx; ++b) {
    dist_ac[b] = dist[b];
    dist_rel_ac[b] = rel[b];
  }
  int b = 2;
  for (int64_t low = 2; low < mx; low *= 2, ++b)
    for (int64_t d = low; d < 2 * low && d <= mx; ++d) {
      dist_ac[b] += dist[d];
      dist_rel_ac[b] += rel[d];
    }
  free(dist);
  free(rel);
  return 0;
}
