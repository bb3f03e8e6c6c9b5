/*
 * ORACLE — test infrastructure only.  A driver for the reference's own CPU
 * reductions, compiled by oracle/Makefile straight from the reference's
 * source files where they lie (src/cuda/functions_host.cu,
 * src/cuda/algorithms/kernels_host.cu, algorithms/standard/standard.cu,
 * algorithms/twist/twist.cu, algorithms/ph_row/ph_row.cu).  Nothing of the
 * reference is copied here: this file supplies the three stubs those sources
 * need outside CUDA/MATLAB (the event type, tic/toc and the O(m) per-column
 * progress tracker) and rebuilds on the host what src/cuda/openph.cu:29-170
 * prepares before dispatch (slot store, low, dimension lists).
 *
 *   ref_ph <algstr> <col_width> <in.csc> <out.bin>
 *
 * algstr is one of standard, twist, ph_row.  in.csc is the canonical CSC file
 * ("OPHCSC01", int64 m, int64 nnz, int64 colptr[m+1], int32 rows[nnz]);
 * out.bin receives int32 low[m] (0-based, -1 = zero column), int32 ess[m],
 * int32 num_iters and a double with the wall seconds of the reduction call.
 * A slot overflow inside the reference ends the process (the reference calls
 * exit(0) at kernels_host.cu:23), which the caller sees as a missing output.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iostream>
using namespace std;

typedef int cudaEvent_t;
static inline void tic(cudaEvent_t *, cudaEvent_t *) {}
static inline void toc(cudaEvent_t, cudaEvent_t, float *) {}
static inline void track_host(int, int, int *, int *, int *, int *, int *, float *, float *, float *,
                              float *, float *, float *, float) {}

#include "functions_host.cu"
#include "algorithms/kernels_host.cu"
#include "algorithms/standard/standard.cu"
#include "algorithms/twist/twist.cu"
#include "algorithms/ph_row/ph_row.cu"

static double now_s() {
    timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
    if (argc != 5) { fprintf(stderr, "usage: ref_ph algstr col_width in.csc out.bin\n"); return 2; }
    const char *alg = argv[1];
    int col_width = atoi(argv[2]);
    FILE *f = fopen(argv[3], "rb");
    if (!f) return 3;
    char magic[8]; int64_t m64, nnz64;
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "OPHCSC01", 8) != 0) return 3;
    if (fread(&m64, 8, 1, f) != 1 || fread(&nnz64, 8, 1, f) != 1) return 3;
    int m = (int)m64;
    int64_t *colptr = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
    int *rows = (int *)malloc(sizeof(int) * (nnz64 ? nnz64 : 1));
    if (fread(colptr, 8, m + 1, f) != (size_t)(m + 1)) return 3;
    if (nnz64 && fread(rows, 4, nnz64, f) != (size_t)nnz64) return 3;
    fclose(f);

    /* p = col_width * max column nnz (src/cuda/openph.cu:41) */
    int maxnnz = 0;
    for (int j = 0; j < m; j++) { int n = (int)(colptr[j + 1] - colptr[j]); if (n > maxnnz) maxnnz = n; }
    int p = col_width * maxnnz; if (p < 1) p = 1;
    int64_t mp = (int64_t)m * p;
    int *rows_mp = (int *)malloc(sizeof(int) * mp), *aux_mp = (int *)malloc(sizeof(int) * mp);
    int *low = (int *)malloc(sizeof(int) * m), *arglow = (int *)malloc(sizeof(int) * m);
    int *classes = (int *)malloc(sizeof(int) * m), *ess = (int *)malloc(sizeof(int) * m);
    int *low_true = (int *)calloc(m, sizeof(int)), *ess_true = (int *)calloc(m, sizeof(int));
    float *float_m = (float *)calloc(m, sizeof(float));
    float *e1 = (float *)calloc(m + 1, sizeof(float)), *e2 = (float *)calloc(m + 1, sizeof(float));
    float *e3 = (float *)calloc(m + 1, sizeof(float)), *e4 = (float *)calloc(m + 1, sizeof(float));
    float *tt = (float *)calloc(m + 1, sizeof(float));
    if (!rows_mp || !aux_mp) return 4;
    for (int64_t i = 0; i < mp; i++) { rows_mp[i] = -1; aux_mp[i] = -1; }
    for (int j = 0; j < m; j++) {
        int n = (int)(colptr[j + 1] - colptr[j]);
        for (int k = 0; k < n; k++) rows_mp[(int64_t)j * p + k] = rows[colptr[j] + k];
        low[j] = n ? rows[colptr[j + 1] - 1] : -1;
        arglow[j] = -1; classes[j] = 0; ess[j] = 1;
    }
    /* dimension lists as src/cuda/dimensions.cu:54-112 builds them */
    int *dim = (int *)malloc(sizeof(int) * m), *dim_order = (int *)malloc(sizeof(int) * m);
    int *dim_next = (int *)malloc(sizeof(int) * m);
    int complex_dim = -1;
    for (int j = 0; j < m; j++) { dim[j] = (int)(colptr[j + 1] - colptr[j]) - 1; if (dim[j] > complex_dim) complex_dim = dim[j]; }
    int cdim = complex_dim + 2;
    int *dim_start = (int *)malloc(sizeof(int) * cdim), *last = (int *)malloc(sizeof(int) * cdim);
    int *count = (int *)calloc(cdim, sizeof(int));
    for (int c = 0; c < cdim; c++) { dim_start[c] = -1; last[c] = -1; }
    for (int j = 0; j < m; j++) {
        int c = dim[j] + 1;
        dim_order[j] = count[c]++;
        dim_next[j] = -1;
        if (last[c] > -1) dim_next[last[c]] = j;
        last[c] = j;
        if (dim_order[j] == 0) dim_start[c] = j;
    }
    int iters = 0;
    double t0 = now_s();
    if (strcmp(alg, "twist") == 0)
        twist(low, arglow, classes, ess, rows_mp, m, p, dim, dim_order, dim_next, dim_start, complex_dim,
              aux_mp, low_true, ess_true, float_m, e1, e2, e3, e4, tt, &iters);
    else if (strcmp(alg, "standard") == 0)
        standard(low, arglow, classes, ess, rows_mp, m, p, aux_mp, low_true, ess_true, float_m, e1, e2, e3, e4,
                 tt, &iters);
    else if (strcmp(alg, "ph_row") == 0)
        ph_row(low, arglow, classes, ess, rows_mp, m, p, dim, dim_order, dim_next, dim_start, aux_mp, low_true,
               ess_true, float_m, e1, e2, e3, e4, tt, &iters);
    else { fprintf(stderr, "Not recognised\n"); return 5; }
    double secs = now_s() - t0;
    FILE *o = fopen(argv[4], "wb");
    if (!o) return 6;
    fwrite(low, 4, m, o); fwrite(ess, 4, m, o); fwrite(&iters, 4, 1, o); fwrite(&secs, 8, 1, o);
    fclose(o);
    return 0;
}
