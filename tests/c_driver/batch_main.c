/* A C caller of the batch API (include/hbicg.h): one family per Matrix Market
 * file (loaded with the reference's csr_load_matrix; sigma[i] = (i + 1) (0.01
 * / m), b = 1, seed 0), all solved by one hbicg_batch_solve_opts call with the
 * default options (the small families in the shared persistent launch, the
 * others on the host workers).  It includes only the headers in include/ and
 * links only libhbicg.so.
 *
 * usage: batch_main <m> <out.bin> <a.mtx> [<b.mtx> ...]
 * out.bin, per family: int32 status, int32 k, int32 rows, then x (m * rows
 * doubles, shift-major). */
#include <stdio.h>
#include <stdlib.h>

#include "hbicg.h"
#include "matrix.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s m out.bin a.mtx [b.mtx ...]\n", argv[0]);
        return 2;
    }
    const int m = atoi(argv[1]);
    const int nf = argc - 3;
    CSR_Matrix *A = (CSR_Matrix *)calloc((size_t)nf, sizeof(CSR_Matrix));
    hbicg_family *F = (hbicg_family *)calloc((size_t)nf, sizeof(hbicg_family));
    double *sigma = (double *)malloc(sizeof(double) * (size_t)m);
    if (!A || !F || !sigma || m < 1) return 2;
    for (int i = 0; i < m; ++i) sigma[i] = (i + 1) * (0.01 / m);
    for (int f = 0; f < nf; ++f) {
        csr_init_matrix(&A[f]);
        csr_load_matrix(argv[3 + f], &A[f]);
        const unsigned n = A[f].rows;
        double *b = (double *)malloc(sizeof(double) * n);
        double *x = (double *)calloc((size_t)n * (size_t)m, sizeof(double));
        if (!b || !x) return 2;
        for (unsigned i = 0; i < n; ++i) b[i] = 1.0;
        F[f].n = n;
        F[f].nnz = A[f].nz;
        F[f].ptr = A[f].ptr;
        F[f].col = A[f].col;
        F[f].val = A[f].val;
        F[f].b = b;
        F[f].sigma = sigma;
        F[f].m = m;
        F[f].seed = 0;
        F[f].x = x;
    }
    hbicg_params p;
    hbicg_params_default(&p);
    p.tol = 1e-10;
    p.max_iter = 5000;
    p.refine = 0;
    hbicg_batch_opts o;
    hbicg_batch_opts_default(&o);
    o.workers = 2;
    double wall_ms = 0.0;
    const int rc = hbicg_batch_solve_opts(F, nf, &p, &o, &wall_ms);
    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    for (int f = 0; f < nf; ++f) {
        const int head[3] = {F[f].status, F[f].k, (int)F[f].n};
        fwrite(head, sizeof(int), 3, out);
        fwrite(F[f].x, sizeof(double), (size_t)F[f].n * (size_t)m, out);
        printf("family %d: n %u status %d k %d\n", f, F[f].n, F[f].status, F[f].k);
    }
    fclose(out);
    printf("batch status %d, %.1f ms\n", rc, wall_ms);
    return rc == HBICG_OK ? 0 : 1;
}
