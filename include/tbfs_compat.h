/*
 * tbfs_compat.h -- drop-in replacements for the reference's GPU BFS entry
 * points, with the reference's exact C signatures.
 *
 * Each call behaves like the function it replaces: it takes host arrays,
 * allocates device memory, uploads the graph, runs the BFS `repetition`
 * times and copies the result of the last run back into the caller's host
 * arrays.  Output conventions follow each reference variant:
 *
 *   td_csc  : S[v] = depth, root and unreached vertices = 0;
 *             sigma (float) = path count rounded to float.
 *   bu_csc  : S[v] = depth, root = 0, unreached = -1.
 *   tdbu_csc: S as bu_csc; sigma (int32, two's-complement wrap) holds the
 *             path count for vertices the reference reaches in its top-down
 *             levels and 0 for those it reaches bottom-up.  The reference
 *             stays top-down while the last level found at most 0.001*n
 *             vertices (float compare) and never switches back.
 *   td_cooc : sigma (float) only.
 *
 * Differences, all on inputs where the reference itself is not defined:
 *   - the return value is 0 on success and a tbfs_status code on failure
 *     (the reference returns 0 or exits the process from checkCudaErrors);
 *   - an out-of-range root or negative size is rejected, not dereferenced;
 *   - path counts are exact up to INT64_MAX before narrowing, so vertices
 *     whose int32 count wraps to <= 0 in the reference kernels (which then
 *     mislabel S) get their true depth here;
 *   - `bbreak` only changes the reference's speed, never its result, and is
 *     accepted but not needed: bottom-up levels here always stop at the
 *     first parent found.
 * _sc and _wa select the same GB300 engine: the reference's thread- versus
 * warp-per-column split is a tuning choice the engine makes per level.
 */
#ifndef TBFS_COMPAT_H
#define TBFS_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

/* replaces TurboBFS_CSC_TD/bfstdcsc.h:54-55 (bfsgputdcsc_sc.cu:47-149) */
int bfs_gpu_td_csc_sc(int *IC_h, int *CP_h, int *S_h, float *sigma_h, int r,
                      int nz, int n, int repetition);

/* replaces TurboBFS_CSC_TD/bfstdcsc.h:65-66 (bfsgputdcsc_wa.cu:46-150) */
int bfs_gpu_td_csc_wa(int *IC_h, int *CP_h, int *S_h, float *sigma_h, int r,
                      int nz, int n, int repetition);

/* replaces TurboBFS_CSC_BU/bfsbucsc.h:55-56 (bfsgpubucsc_sc.cu:47-114) */
int bfs_gpu_bu_csc_sc(int *I_h, int *CP_h, int *S_h, int r, int nz, int n,
                      int repetition, int bbreak);

/* replaces TurboBFS_CSC_BU/bfsbucsc.h:66-67 (bfsgpubucsc_wa.cu:46-113) */
int bfs_gpu_bu_csc_wa(int *I_h, int *CP_h, int *S_h, int r, int nz, int n,
                      int repetition, int bbreak);

/* replaces TurboBFS_CSC_TDBU/bfstdbucsc.h:56-57 (bfsgputdbucsc_sc.cu:53-186) */
int bfs_gpu_tdbu_csc_sc(int *I_h, int *CP_h, int *S_h, int *sigma_h, int r,
                        int nz, int n, int repetition, int bbreak);

/* replaces TurboBFS_CSC_TDBU/bfstdbucsc.h:67-68 (bfsgputdbucsc_wa.cu:54-191) */
int bfs_gpu_tdbu_csc_wa(int *IC_h, int *CP_h, int *S_h, int *sigma_h, int r,
                        int nz, int n, int repetition, int bbreak);

/* replaces TurboBFS_COOC_TD/bfstdcooc.h:48-49 (bfsgputdcooc_sc.cu:44-140) */
int bfs_gpu_td_cooc_sc(int *I_h, int *J_h, float *sigma_h, int r, int nz,
                       int n, int repetition);

#ifdef __cplusplus
}
#endif
#endif /* TBFS_COMPAT_H */
