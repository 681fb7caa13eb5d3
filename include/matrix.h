/* Sparse matrix types and loaders, GB300 solver edition.
 *
 * Drop-in for the reference's src/matrix.h:10-56 with single-rank semantics:
 * the structs keep the reference's exact field order and types so that
 * caller code and binary layouts are unchanged; <mpi.h> is not included (one
 * process drives one GPU).  The MPI_* functions keep their names and behave as
 * the reference does on one rank: the "diagonal block" is the whole matrix and
 * the "off-diagonal block" is empty.
 *
 * Products (mult, mult_block, MPI_csr_spmv_ovlap, MPI_csr_spmv_async) run on
 * the GPU: host arrays are copied to the device, multiplied by the solver's
 * CSR SpMV kernel and copied back.  Loading and COO->CSR conversion run on
 * the host while reading the file.
 */
#ifndef MATRIX_H
#define MATRIX_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mmio.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double *val;       /* nonzero values */
    unsigned int *row; /* row index of each nonzero (0-based) */
    unsigned int *col; /* column index of each nonzero (0-based) */
    unsigned int nz;   /* number of nonzeros */
    unsigned int rows;
    unsigned int cols;
} COO_Matrix;

typedef struct {
    double *val;       /* nonzero values, row by row */
    unsigned int *col; /* column index of each nonzero (0-based) */
    unsigned int *ptr; /* rows+1 offsets into val/col */
    unsigned int nz;
    unsigned int rows;
    unsigned int cols;
} CSR_Matrix;

typedef struct {
    unsigned int nz, rows, cols; /* global sizes */
    MM_typecode code;            /* Matrix Market typecode of the source file */
    int *recvcounts;             /* rows per rank (one entry here) */
    int *displs;                 /* first row per rank (one entry here) */
} INFO_Matrix;

/* src/matrix.h:35-42 */
void coo_init_matrix(COO_Matrix *m);
void coo_free_matrix(COO_Matrix *m);
int coo_load_matrix(char *filename, COO_Matrix *coo);
void coo_copy(COO_Matrix *in, COO_Matrix *out);
void coo_reorder_by_rows(COO_Matrix *m);
void coo_merge(unsigned int *A, unsigned int *A2, double *A3, unsigned int *B, unsigned int *B2, double *B3, int left,
               int mid, int right);
void coo_merge_sort(unsigned int *A, unsigned int *A2, double *A3, unsigned int *B, unsigned int *B2, double *B3,
                    int left, int right);

/* src/matrix.h:44-47 */
void csr_init_matrix(CSR_Matrix *m);
void csr_free_matrix(CSR_Matrix *m);
void coo2csr(COO_Matrix *in, CSR_Matrix *out);
int csr_load_matrix(char *filename, CSR_Matrix *m);

/* src/matrix.h:49-54 (single rank) */
void MPI_coo_load_matrix_block(char *filename, COO_Matrix *matrix_loc_diag, COO_Matrix *matrix_loc_offd,
                               INFO_Matrix *matrix_info);
void MPI_csr_load_matrix_block(char *filename, CSR_Matrix *matrix_loc_diag, CSR_Matrix *matrix_loc_offd,
                               INFO_Matrix *matrix_info);
void MPI_csr_spmv_ovlap(CSR_Matrix *matrix_loc_diag, CSR_Matrix *matrix_loc_offd, INFO_Matrix *matrix_info,
                        double *x_loc, double *x, double *y_loc);
void MPI_csr_spmv_async(CSR_Matrix *matrix_loc_diag, CSR_Matrix *matrix_loc_offd, INFO_Matrix *matrix_info,
                        double *x_loc, double **x_recv, double *y_loc, int numsend, int myid, int *recv_procs);
void mult(CSR_Matrix *A_loc, double *x, double *y_loc);
void mult_block(CSR_Matrix *A_loc, double *x_part, double *y_loc, int start_index, int end_index);

/* src/matrix.h:56 */
void csr_shift_diagonal(CSR_Matrix *A_diag, double sigma);

#ifdef __cplusplus
}
#endif
#endif /* MATRIX_H */
