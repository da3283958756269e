/*
 * tbfs_oracle.h -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the
 * reference TurboBFS algorithms, used by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg as the checker.  The product library never
 * links, loads or calls anything here.
 *
 * Parity pinning: every oracle_seq_* function is checked bit-for-bit against
 * the reference's own sequential sources compiled unchanged from the
 * reference tree (oracle/Makefile target `ref`, outputs in oracle/_ref/) on
 * all reference fixtures, and the results are frozen as golden vectors in
 * tests/golden/.
 */
#ifndef TBFS_ORACLE_H
#define TBFS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Sequential top-down BFS over CSC with float sigma
 * (TurboBFS_CSC_TD/bfstdcsc_seq.c:27-96, spmvcsc_seq.c:22-41,
 * bfstdcsc_seq_utils.c:21-103).  init_S = 0: S is left as passed in (the
 * CSC_TD driver passes zeros, bfstdcsc_main.c:136); init_S = 1: S = -1 and
 * S[r] = 0 first (TurboBFS_CSC_BU/bfstdcsc_seq.c:26-36).  sigma must be
 * zeroed by the caller, as the drivers' calloc does.  Returns the level
 * count d printed by the reference. */
int oracle_seq_csc_f32(const int *IC, const int *CP, int *S, float *sigma, int r,
                       int nz, int n, int init_S);

/* Same algebra with int32 f and sigma (TurboBFS_CSC_TDBU/bfstdcsc_seq.c:26-96
 * and its bfstdcsc_seq_utils.c); int32 sums wrap in two's complement. */
int oracle_seq_csc_i32(const int *IC, const int *CP, int *S, int *sigma, int r,
                       int nz, int n);

/* Sequential top-down BFS over COOC, float sigma, f_t never cleared
 * (TurboBFS_COOC_TD/bfstdcooc_seq.c:29-91, spmvcooc_seq.c:27-36). */
int oracle_seq_cooc_f32(const int *I, const int *J, float *sigma, int r, int nz,
                        int n);

/* Exact BFS: S (-1 unreached) and sigma as the true path count when it is
 * below 2^63; ovf[v] = 1 marks vertices whose count is >= 2^63 (sigma[v] is
 * then -1).  Counts are carried in saturating 128-bit integers.  Returns
 * the number of non-empty levels. */
int oracle_exact_bfs(const int *CP, const int *IC, int n, int r, int *S,
                     int64_t *sigma, uint8_t *ovf);

/* Emulations of what each reference GPU driver hands back (sequential
 * restatement of the kernels; their results do not depend on thread order):
 *  td_csc  : bfsgputdcsc_sc.cu:159-208 (and _wa.cu:159-219): int32 f with
 *            wrap, float sigma += ft, S zero-initialised;
 *  bu_csc  : bfsgpubucsc_sc.cu:122-148: S only, -1 initialised;
 *  tdbu_csc: bfsgputdbucsc_sc.cu:53-278: host switch to bottom-up once a
 *            top-down level found more than 0.001*n vertices (float), int32
 *            sigma updated in top-down levels only;
 *  td_cooc : bfsgputdcooc_sc.cu:94-188: edge-parallel int32 atomics, float
 *            sigma, no S. */
int oracle_gpu_td_csc(const int *IC, const int *CP, int *S, float *sigma, int r,
                      int nz, int n);
int oracle_gpu_bu_csc(const int *IC, const int *CP, int *S, int r, int nz, int n);
int oracle_gpu_tdbu_csc(const int *IC, const int *CP, int *S, int *sigma, int r,
                        int nz, int n, int *switch_level);
int oracle_gpu_td_cooc(const int *I, const int *J, float *sigma, int r, int nz,
                       int n);

/* CPU baseline: oracle_seq_csc_i32 from k roots on `threads` host threads,
 * each BFS single-threaded.  seconds[i] = wall time of root i's BFS;
 * edges[i] = sum of column lengths over the vertices it reached.  Returns
 * the wall time of the whole batch in seconds. */
double oracle_seq_many(const int *IC, const int *CP, int nz, int n,
                       const int *roots, int k, int threads, double *seconds,
                       int64_t *edges);

/* Brandes betweenness with the GPU sweep's summation order (see .c) */
int oracle_brandes(const int *orp, const int *ojr, int n, const int *roots, int k, double *bc);

/* Degree statistics of a degree vector deg[n], as the reference's drivers
 * compute them (TurboBFS_CSC_TD/degree.c:36-141, called from
 * bfstdcsc_main.c:177-195): the maximum and the first vertex holding it
 * (*argmax = -1 when every degree is 0; the reference leaves it unset), the
 * mean (sum in int64 here; the reference's int sum wraps past 2^31) and the
 * sample standard deviation (divisor n - 1), and the accumulated log2
 * distribution: dist_ac[0] / dist_ac[1] = vertices of degree 0 / 1 and
 * dist_ac[b] (b >= 2) = vertices with degree in [2^(b-1), 2^b) while
 * 2^(b-1) < max -- so a maximum that is a power of two is counted in no
 * bucket, as in degree_dist_ac -- with dist_rel_ac the same sums of the
 * per-degree percentages 100 * count / n.  cap = entries of dist_ac and
 * dist_rel_ac (unused buckets are 0).  Returns 0, or -1 when cap is too
 * small for max. */
int oracle_degree_stats(const int *deg, int n, int64_t *maxd, int64_t *argmax, double *mean,
                        double *sd, int64_t *dist_ac, double *dist_rel_ac, int cap);

#ifdef __cplusplus
}
#endif
#endif
