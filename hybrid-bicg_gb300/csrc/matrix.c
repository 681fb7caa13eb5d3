/* COO/CSR types, Matrix Market loaders and products (include/matrix.h).
 *
 * Semantics follow the reference on one rank (src/matrix.c):
 *   - indices are converted to 0-based while reading (:86-87, :333-334);
 *   - COO->CSR orders entries by row with a stable sort, so each row keeps the
 *     file's order (:176-232).  Here that is a counting sort by row;
 *   - symmetric files are not expanded (the reference returns the flag,
 *     :93, and its row-block loader ignores it);
 *   - the row-block loader puts every entry with a column inside the rank's
 *     row range into the diagonal block; on one rank that is every entry of a
 *     square matrix (:336-340).
 * Deliberate difference: for integer and pattern files the row-block loader
 * stores the integer value / 1.0, where the reference leaves the value it
 * last parsed (:316-331, :384); real files load identically.
 * Errors print the reference's messages and exit, as the reference does.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "host_internal.h"
#include "matrix.h"

static void die(const char *msg) {
    fprintf(stderr, "%s", msg);
    exit(EXIT_FAILURE);
}

void coo_init_matrix(COO_Matrix *m) {
    m->val = NULL;
    m->row = m->col = NULL;
    m->nz = m->rows = m->cols = 0;
}

void coo_free_matrix(COO_Matrix *m) {
    free(m->val);
    free(m->row);
    free(m->col);
    coo_init_matrix(m);
}

/* Reads the banner and size line and checks for a coordinate matrix. */
static FILE *open_mtx(const char *filename, MM_typecode *code, int *M, int *N, int *nz) {
    FILE *f = fopen(filename, "r");
    if (!f) {
        fprintf(stderr, "ERROR: can't open file \"%s\"\n", filename);
        exit(EXIT_FAILURE);
    }
    if (mm_read_banner(f, code) != 0) die("ERROR: Could not process Matrix Market banner.\n");
    if (!mm_is_matrix(*code) || !mm_is_sparse(*code) || !mm_is_coordinate(*code)) {
        char *s = mm_typecode_to_str(*code);
        fprintf(stderr, "Sorry, this application does not support Market Market type: [%s]\n", s ? s : "?");
        free(s);
        exit(EXIT_FAILURE);
    }
    if (mm_read_mtx_crd_size(f, M, N, nz) != 0) die("ERROR: Could not read matrix size.\n");
    return f;
}

/* one triplet; 0-based row/col; pattern -> 1.0, integer -> its value */
static void read_entry(FILE *f, MM_typecode code, unsigned *row, unsigned *col, double *val) {
    int r, c, iv;
    double v = 1.0;
    if (mm_is_pattern(code)) {
        if (fscanf(f, "%d %d", &r, &c) < 2) die("ERROR: reading matrix data.\n");
    } else if (mm_is_integer(code)) {
        if (fscanf(f, "%d %d %d", &r, &c, &iv) < 3) die("ERROR: reading matrix data.\n");
        v = (double)iv;
    } else {
        if (fscanf(f, "%d %d %lg", &r, &c, &v) < 3) die("ERROR: reading matrix data.\n");
    }
    *row = (unsigned)(r - 1);
    *col = (unsigned)(c - 1);
    *val = v;
}

/* The reference's loader (src/matrix.c:26-94): same entries, same values,
 * same exit on a bad file; the parsing runs on all host cores
 * (hbicg_mm_read).  Returns whether the file is stored as symmetric. */
int coo_load_matrix(char *filename, COO_Matrix *coo) {
    hbicg_coo c;
    if (hbicg_mm_read(filename, 0, 0, &c) != HBICG_OK) {
        fprintf(stderr, "ERROR: %s\n", hbicg_last_message());
        exit(EXIT_FAILURE);
    }
    coo->rows = c.rows;
    coo->cols = c.cols;
    coo->nz = (unsigned)c.nnz;
    coo->val = c.val;
    coo->row = c.row;
    coo->col = c.col;
    return c.symmetry == 1;
}

void coo_copy(COO_Matrix *in, COO_Matrix *out) {
    out->nz = in->nz;
    out->rows = in->rows;
    out->cols = in->cols;
    out->val = malloc(sizeof(double) * ((size_t)in->nz + 1));
    out->row = malloc(sizeof(unsigned) * ((size_t)in->nz + 1));
    out->col = malloc(sizeof(unsigned) * ((size_t)in->nz + 1));
    memcpy(out->val, in->val, sizeof(double) * in->nz);
    memcpy(out->row, in->row, sizeof(unsigned) * in->nz);
    memcpy(out->col, in->col, sizeof(unsigned) * in->nz);
}

/* Stable merge of A[left..mid] and A[mid+1..right] (keys A, payloads A2, A3)
 * through the scratch arrays B*; equal keys keep their order. */
void coo_merge(unsigned int *A, unsigned int *A2, double *A3, unsigned int *B, unsigned int *B2, double *B3, int left,
               int mid, int right) {
    int a = left, b = mid + 1, o = left;
    while (a <= mid || b <= right) {
        int take_a = b > right || (a <= mid && A[a] <= A[b]);
        int src = take_a ? a++ : b++;
        B[o] = A[src];
        B2[o] = A2[src];
        B3[o] = A3[src];
        o++;
    }
    memcpy(A + left, B + left, sizeof(unsigned) * (size_t)(right - left + 1));
    memcpy(A2 + left, B2 + left, sizeof(unsigned) * (size_t)(right - left + 1));
    memcpy(A3 + left, B3 + left, sizeof(double) * (size_t)(right - left + 1));
}

/* Stable sort of [left, right] by A (bottom-up merge passes). */
void coo_merge_sort(unsigned int *A, unsigned int *A2, double *A3, unsigned int *B, unsigned int *B2, double *B3,
                    int left, int right) {
    for (int w = 1; left + w <= right; w *= 2)
        for (int lo = left; lo + w <= right; lo += 2 * w) {
            int mid = lo + w - 1, hi = lo + 2 * w - 1;
            if (hi > right) hi = right;
            coo_merge(A, A2, A3, B, B2, B3, lo, mid, hi);
        }
}

/* Stable counting sort by row. */
void coo_reorder_by_rows(COO_Matrix *m) {
    const unsigned nz = m->nz;
    unsigned maxr = m->rows;
    for (unsigned i = 0; i < nz; i++)
        if (m->row[i] >= maxr) maxr = m->row[i] + 1;
    unsigned *cnt = calloc((size_t)maxr + 1, sizeof(unsigned));
    unsigned *r2 = malloc(sizeof(unsigned) * ((size_t)nz + 1)), *c2 = malloc(sizeof(unsigned) * ((size_t)nz + 1));
    double *v2 = malloc(sizeof(double) * ((size_t)nz + 1));
    for (unsigned i = 0; i < nz; i++) cnt[m->row[i] + 1]++;
    for (unsigned r = 0; r < maxr; r++) cnt[r + 1] += cnt[r];
    for (unsigned i = 0; i < nz; i++) {
        unsigned d = cnt[m->row[i]]++;
        r2[d] = m->row[i];
        c2[d] = m->col[i];
        v2[d] = m->val[i];
    }
    free(m->row);
    free(m->col);
    free(m->val);
    m->row = r2;
    m->col = c2;
    m->val = v2;
    free(cnt);
}

void csr_init_matrix(CSR_Matrix *m) {
    m->val = NULL;
    m->col = m->ptr = NULL;
    m->nz = m->rows = m->cols = 0;
}

void csr_free_matrix(CSR_Matrix *m) {
    free(m->val);
    free(m->col);
    free(m->ptr);
    csr_init_matrix(m);
}

void coo2csr(COO_Matrix *in, CSR_Matrix *out) {
    COO_Matrix t;
    coo_copy(in, &t);
    coo_reorder_by_rows(&t);
    out->nz = in->nz;
    out->rows = in->rows;
    out->cols = in->cols;
    out->val = malloc(sizeof(double) * ((size_t)in->nz + 1));
    out->col = malloc(sizeof(unsigned) * ((size_t)in->nz + 1));
    out->ptr = malloc(sizeof(unsigned) * ((size_t)in->rows + 1));
    unsigned e = 0;
    out->ptr[0] = 0;
    for (unsigned r = 0; r < in->rows; r++) {
        while (e < t.nz && t.row[e] == r) {
            out->val[e] = t.val[e];
            out->col[e] = t.col[e];
            e++;
        }
        out->ptr[r + 1] = e;
    }
    coo_free_matrix(&t);
}

int csr_load_matrix(char *filename, CSR_Matrix *m) {
    COO_Matrix t;
    coo_init_matrix(&t);
    int sym = coo_load_matrix(filename, &t);
    coo2csr(&t, m);
    coo_free_matrix(&t);
    return sym;
}

void MPI_coo_load_matrix_block(char *filename, COO_Matrix *diag, COO_Matrix *offd, INFO_Matrix *info) {
    MM_typecode code;
    int M, N, nz;
    FILE *f = open_mtx(filename, &code, &M, &N, &nz);
    info->nz = (unsigned)nz;
    info->rows = (unsigned)M;
    info->cols = (unsigned)N;
    memcpy(info->code, code, sizeof(MM_typecode));
    if (info->recvcounts) info->recvcounts[0] = M;
    if (info->displs) info->displs[0] = 0;
    unsigned *row = malloc(sizeof(unsigned) * ((size_t)nz + 1)), *col = malloc(sizeof(unsigned) * ((size_t)nz + 1));
    double *val = malloc(sizeof(double) * ((size_t)nz + 1));
    unsigned nd = 0, no = 0;
    for (int i = 0; i < nz; i++) {
        read_entry(f, code, &row[i], &col[i], &val[i]);
        if (row[i] < (unsigned)M) {
            if (col[i] < (unsigned)M) nd++;
            else no++;
        }
    }
    fclose(f);
    coo_init_matrix(diag);
    coo_init_matrix(offd);
    diag->rows = diag->cols = (unsigned)M;
    offd->rows = (unsigned)M;
    offd->cols = (unsigned)N;
    diag->nz = nd;
    offd->nz = no;
    diag->row = malloc(sizeof(unsigned) * ((size_t)nd + 1));
    diag->col = malloc(sizeof(unsigned) * ((size_t)nd + 1));
    diag->val = malloc(sizeof(double) * ((size_t)nd + 1));
    offd->row = malloc(sizeof(unsigned) * ((size_t)no + 1));
    offd->col = malloc(sizeof(unsigned) * ((size_t)no + 1));
    offd->val = malloc(sizeof(double) * ((size_t)no + 1));
    unsigned a = 0, b = 0;
    for (int i = 0; i < nz; i++) {
        if (row[i] >= (unsigned)M) continue;
        if (col[i] < (unsigned)M) {
            diag->row[a] = row[i];
            diag->col[a] = col[i];
            diag->val[a++] = val[i];
        } else {
            offd->row[b] = row[i];
            offd->col[b] = col[i];
            offd->val[b++] = val[i];
        }
    }
    free(row);
    free(col);
    free(val);
}

void MPI_csr_load_matrix_block(char *filename, CSR_Matrix *diag, CSR_Matrix *offd, INFO_Matrix *info) {
    COO_Matrix cd, co;
    MPI_coo_load_matrix_block(filename, &cd, &co, info);
    csr_init_matrix(diag);
    coo2csr(&cd, diag);
    csr_init_matrix(offd);
    coo2csr(&co, offd);
    coo_free_matrix(&cd);
    coo_free_matrix(&co);
}

static void spmv_or_die(const CSR_Matrix *A, const double *x, double *y, int accumulate) {
    int rc = hbicg__host_spmv(A->rows, A->cols, A->ptr ? A->ptr[A->rows] : 0, A->ptr, A->col, A->val, x, y,
                              accumulate);
    if (rc) {
        fprintf(stderr, "hbicg: SpMV failed: %s (%s)\n", hbicg_status_string(rc), hbicg_last_message());
        exit(EXIT_FAILURE);
    }
}

/* y_loc += A x (src/matrix.c:498-516), on the GPU */
void mult(CSR_Matrix *A_loc, double *x, double *y_loc) { spmv_or_die(A_loc, x, y_loc, 1); }

/* y_loc += A restricted to columns [start, end), x_part indexed from start
 * (src/matrix.c:522-533), on the GPU through a zero-padded x */
void mult_block(CSR_Matrix *A_loc, double *x_part, double *y_loc, int start_index, int end_index) {
    double *xf = calloc((size_t)A_loc->cols + 1, sizeof(double));
    for (int i = start_index; i < end_index && i < (int)A_loc->cols; i++) xf[i] = x_part[i - start_index];
    spmv_or_die(A_loc, xf, y_loc, 1);
    free(xf);
}

/* y_loc = A_diag x_loc + A_offd x with x the gathered vector; on one rank the
 * gather copies x_loc into x (src/matrix.c:428-441) */
void MPI_csr_spmv_ovlap(CSR_Matrix *diag, CSR_Matrix *offd, INFO_Matrix *info, double *x_loc, double *x,
                        double *y_loc) {
    const int off = info->displs ? info->displs[0] : 0;
    if (x && x != x_loc) memmove(x + off, x_loc, sizeof(double) * diag->rows);
    spmv_or_die(diag, x_loc, y_loc, 0);
    if (offd && offd->nz && offd->ptr) spmv_or_die(offd, x ? x : x_loc, y_loc, 1);
}

/* single rank: no messages, y_loc = A_diag x_loc (src/matrix.c:450-492) */
void MPI_csr_spmv_async(CSR_Matrix *diag, CSR_Matrix *offd, INFO_Matrix *info, double *x_loc, double **x_recv,
                        double *y_loc, int numsend, int myid, int *recv_procs) {
    (void)offd;
    (void)info;
    (void)x_recv;
    (void)numsend;
    (void)myid;
    (void)recv_procs;
    spmv_or_die(diag, x_loc, y_loc, 0);
}

void csr_shift_diagonal(CSR_Matrix *A, double sigma) {
    for (unsigned i = 0; i < A->rows; i++) {
        int found = 0;
        for (unsigned e = A->ptr[i]; e < A->ptr[i + 1]; e++)
            if (A->col[e] == i) {
                A->val[e] += sigma;
                found = 1;
                break;
            }
        if (!found) {
            fprintf(stderr, "Error: Diagonal element not found in row %u.\n", i);
            exit(EXIT_FAILURE);
        }
    }
}
