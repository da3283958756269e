/*
 * tbfs_graphgen.h -- host-side graph construction for the BFS engine:
 * Matrix Market loading with the reference's CSC construction, seeded
 * synthetic generators (Erdos-Renyi, RMAT, perturbed 2-D grid), the
 * symmetrise / drop-self-loop / dedup CSC builder and root selection.
 *
 * All generators are deterministic functions of their arguments (the PRNG
 * is xoshiro256** seeded through splitmix64, both published by Blackman and
 * Vigna) and give identical graphs on every machine and thread count.
 * These calls use no GPU.
 */
#ifndef TBFS_GRAPHGEN_H
#define TBFS_GRAPHGEN_H

#include <stdint.h>
#include "tbfs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Host CSC: col_ptr[n+1], row_idx[nnz]; column v lists the sources u of the
 * edges u->v (the reference's struct Csc, TurboBFS_CSC_TD/bfstdcsc.h:30-34). */
typedef struct tbfs_host_csc {
  int32_t n;
  int32_t reserved;
  int64_t nnz;
  int32_t *col_ptr;
  int32_t *row_idx;
} tbfs_host_csc;

void tbfs_host_csc_free(tbfs_host_csc *g);

/* tbfs_csc_from_edges flags */
#define TBFS_BUILD_SYMMETRIZE 0x1u  /* add v->u for every u->v            */
#define TBFS_BUILD_DROP_LOOPS 0x2u  /* drop u->u                          */
#define TBFS_BUILD_DEDUP 0x4u       /* sort each column, drop repeats     */
#define TBFS_BUILD_SORT 0x8u        /* sort each column (keep repeats)    */

/* Edge k is src[k] -> dst[k]; it lands in column dst[k].  Without SORT or
 * DEDUP the rows of a column keep input order. */
tbfs_status tbfs_csc_from_edges(int32_t n, const int32_t *src, const int32_t *dst,
                                int64_t m, uint32_t flags, tbfs_host_csc **out);

/* Read a Matrix Market coordinate file the way the reference's drivers do
 * (TurboBFS_CSC_TD/bfstdcsc_main.c:106-213 with readMMfilef.c and
 * sparseformatransf.c).  undirected = 1 (the reference's ug=1): every
 * stored entry (i,j) becomes the two CSC entries i->j and j->i, so a stored
 * diagonal entry appears twice in its column.  undirected = 0: entry (i,j)
 * is the edge i->j in column j; columns keep file order.  Values ignored. */
tbfs_status tbfs_mm_read(const char *path, int32_t undirected, tbfs_host_csc **out);

/* G(n, m): m distinct undirected edges without self-loops, symmetric CSC. */
tbfs_status tbfs_gen_er(int32_t n, int64_t m, uint64_t seed, tbfs_host_csc **out);

/* RMAT: 2^scale vertices, edgefactor * 2^scale generated edges, quadrant
 * probabilities a, b, c (d = 1-a-b-c), optional random vertex relabelling,
 * then symmetrised, self-loops dropped, duplicates removed. */
tbfs_status tbfs_gen_rmat(int32_t scale, int32_t edgefactor, double a, double b,
                          double c, uint64_t seed, int32_t permute,
                          tbfs_host_csc **out);

/* side x side 4-neighbour grid (vertex y*side+x); delete_frac of the grid
 * edges removed uniformly; then chord_frac * (remaining edges) chords added
 * between vertices at Manhattan distance 2..max_dist, never raising a degree
 * past max_deg.  Symmetric CSC. */
tbfs_status tbfs_gen_grid(int32_t side, double delete_frac, double chord_frac,
                          int32_t max_dist, int32_t max_deg, uint64_t seed,
                          tbfs_host_csc **out);

/* in_lcc[v] = 1 for the vertices of the largest weakly connected component. */
tbfs_status tbfs_largest_component(const tbfs_host_csc *g, uint8_t *in_lcc,
                                   int64_t *lcc_size);

/* k distinct roots drawn uniformly from the largest component (seeded). */
tbfs_status tbfs_pick_roots(const tbfs_host_csc *g, int32_t k, uint64_t seed,
                            int32_t *roots);

/* Degree profile used as the tuning-cache key: hist[b] = number of vertices
 * whose degree d has floor(log2(d+1)) == b, b < 40; also max and mean. */
tbfs_status tbfs_degree_profile(const tbfs_host_csc *g, int64_t *hist40,
                                int64_t *max_degree, double *mean_degree);

#ifdef __cplusplus
}
#endif
#endif /* TBFS_GRAPHGEN_H */
