/* A caller of the library written the way the reference's driver calls its
 * solver (src/main.c:88-151): load a Matrix Market file with
 * MPI_csr_load_matrix_block, build sigma[i] = (i + 1) (0.01 / sigma_len),
 * r_loc = 1, x_loc_set = 0, call shifted_lopbicg_<variant> with the
 * compile-time EPS and MAX_ITER, and report k.  It includes only the headers
 * in include/ and links only libhbicg.so, so it checks that a reference
 * driver builds and runs against the library unchanged.
 *
 * usage: reference_main <matrix.mtx> <sigma_len> <seed> <dynamic|static|normal> <out.bin>
 * out.bin: int32 k, int32 rows, int32 sigma_len, then x_loc_set (sigma_len * rows doubles,
 * shift-major) and r_loc (rows doubles) as the solver left them. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "matrix.h"
#include "solver.h"
#include "vector.h"

int main(int argc, char **argv) {
    if (argc != 6) {
        fprintf(stderr, "usage: %s matrix.mtx sigma_len seed variant out.bin\n", argv[0]);
        return 2;
    }
    const int sigma_len = atoi(argv[2]);
    const int seed = atoi(argv[3]);
    INFO_Matrix info;
    info.recvcounts = (int *)malloc(sizeof(int));
    info.displs = (int *)malloc(sizeof(int));
    CSR_Matrix *diag = (CSR_Matrix *)malloc(sizeof(CSR_Matrix));
    CSR_Matrix *offd = (CSR_Matrix *)malloc(sizeof(CSR_Matrix));
    csr_init_matrix(diag);
    csr_init_matrix(offd);
    MPI_csr_load_matrix_block(argv[1], diag, offd, &info);
    if (info.cols != info.rows) {
        printf("Error: matrix is not square.\n");
        return 1;
    }
    double *sigma = (double *)malloc(sizeof(double) * (size_t)sigma_len);
    for (int i = 0; i < sigma_len; ++i) sigma[i] = (i + 1) * (0.01 / sigma_len);
    const int rows = (int)diag->rows;
    double *x_loc_set = (double *)malloc(sizeof(double) * (size_t)rows * (size_t)sigma_len);
    double *r_loc = (double *)malloc(sizeof(double) * (size_t)rows);
    for (int i = 0; i < rows; i++) r_loc[i] = 1;
    for (int i = 0; i < rows * sigma_len; i++) x_loc_set[i] = 0;
    int k;
    if (strcmp(argv[4], "static") == 0)
        k = shifted_lopbicg_static(diag, offd, &info, x_loc_set, r_loc, sigma, sigma_len, seed);
    else if (strcmp(argv[4], "normal") == 0)
        k = shifted_lopbicg_normal(diag, offd, &info, x_loc_set, r_loc, sigma, sigma_len, seed);
    else
        k = shifted_lopbicg_dynamic(diag, offd, &info, x_loc_set, r_loc, sigma, sigma_len, seed);
    printf("total_iter: %d\n", k);
    /* the reference's host helpers, as its drivers use them after a solve */
    printf("||r_loc||^2 = %.17g\n", my_ddot(rows, r_loc, r_loc));
    FILE *f = fopen(argv[5], "wb");
    if (!f) return 3;
    const int head[3] = {k, rows, sigma_len};
    fwrite(head, sizeof(int), 3, f);
    fwrite(x_loc_set, sizeof(double), (size_t)rows * (size_t)sigma_len, f);
    fwrite(r_loc, sizeof(double), (size_t)rows, f);
    fclose(f);
    csr_free_matrix(diag);
    csr_free_matrix(offd);
    free(diag);
    free(offd);
    free(info.recvcounts);
    free(info.displs);
    free(sigma);
    free(x_loc_set);
    free(r_loc);
    return k > 0 ? 0 : 4;
}
