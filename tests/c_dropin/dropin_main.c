/*
 * dropin_main.c -- a C caller of the seven drop-in entry points, built the
 * way the reference's driver programs use them (TurboBFS_CSC_TDBU/
 * bfstdbucsc_main.c:127-137,294-305): the CSC and COOC arrays and every
 * output are calloc'd (pageable) host arrays owned by the caller, each call
 * uploads, traverses and copies its result back, and the return value is
 * checked.  It links against libtbfs.so through include/tbfs_compat.h only.
 *
 * usage: dropin_main <in.bin> <out.bin>
 *   in.bin : int32 n, nz, root, bbreak; int32 CP[n+1]; int32 IC[nz]
 *   out.bin: for each entry point in the order below its int32 status, then
 *            its outputs (S int32[n] and/or sigma float32 / int32 [n])
 */
#include <stdio.h>
#include <stdlib.h>

#include "tbfs_compat.h"

static int rd(FILE *f, void *p, size_t sz, size_t cnt) {
  return fread(p, sz, cnt, f) == cnt ? 0 : -1;
}

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[4];
  if (rd(f, hdr, sizeof(int), 4)) return 2;
  const int n = hdr[0], nz = hdr[1], r = hdr[2], bbreak = hdr[3];
  int *CP = (int *)calloc((size_t)n + 1, sizeof(int));
  int *IC = (int *)calloc((size_t)nz + 1, sizeof(int));
  int *J = (int *)calloc((size_t)nz + 1, sizeof(int));
  if (!CP || !IC || !J || rd(f, CP, sizeof(int), (size_t)n + 1) || rd(f, IC, sizeof(int), (size_t)nz))
    return 2;
  fclose(f);
  for (int v = 0; v < n; ++v) /* COOC column of every entry */
    for (int k = CP[v]; k < CP[v + 1]; ++k) J[k] = v;

  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  int *S = (int *)calloc((size_t)n, sizeof(int));
  float *sf = (float *)calloc((size_t)n, sizeof(float));
  int *si = (int *)calloc((size_t)n, sizeof(int));
  int st;

  st = bfs_gpu_td_csc_sc(IC, CP, S, sf, r, nz, n, 1);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o), fwrite(sf, sizeof(float), n, o);
  st = bfs_gpu_td_csc_wa(IC, CP, S, sf, r, nz, n, 1);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o), fwrite(sf, sizeof(float), n, o);
  st = bfs_gpu_bu_csc_sc(IC, CP, S, r, nz, n, 1, bbreak);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o);
  st = bfs_gpu_bu_csc_wa(IC, CP, S, r, nz, n, 1, bbreak);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o);
  st = bfs_gpu_tdbu_csc_sc(IC, CP, S, si, r, nz, n, 1, bbreak);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o), fwrite(si, sizeof(int), n, o);
  st = bfs_gpu_tdbu_csc_wa(IC, CP, S, si, r, nz, n, 1, bbreak);
  fwrite(&st, sizeof st, 1, o), fwrite(S, sizeof(int), n, o), fwrite(si, sizeof(int), n, o);
  st = bfs_gpu_td_cooc_sc(IC, J, sf, r, nz, n, 1);
  fwrite(&st, sizeof st, 1, o), fwrite(sf, sizeof(float), n, o);
  fclose(o);
  free(CP), free(IC), free(J), free(S), free(sf), free(si);
  return 0;
}
