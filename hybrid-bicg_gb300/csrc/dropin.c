/* The reference's solver entry points (src/solver.h:33-35) over the
 * extended API: one-shot solves from host arrays with the reference's
 * argument meaning, return value and error behaviour. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hbicg.h"
#include "solver.h"

/* ------------------------------------------------------------------------ */
/* the reference's entry points (src/solver.h:33-35) */

static double g_tol = EPS;
static int g_maxit = MAX_ITER;
static int g_switching = 1;

void hbicg_dropin_config(double tol, int max_iter, int switching) {
    g_tol = tol;
    g_maxit = max_iter;
    g_switching = switching;
}

/* A_loc_offd holds global column indices (src/matrix.c:387-389); on one rank
 * it is empty.  A non-empty one is merged row by row after the diagonal
 * block's entries. */
static int merged_csr(const CSR_Matrix *d, const CSR_Matrix *o, unsigned **ptr, unsigned **col, double **val) {
    const unsigned n = d->rows;
    const unsigned nz = d->nz + o->nz;
    *ptr = malloc(sizeof(unsigned) * ((size_t)n + 1));
    *col = malloc(sizeof(unsigned) * ((size_t)nz + 1));
    *val = malloc(sizeof(double) * ((size_t)nz + 1));
    if (!*ptr || !*col || !*val) {
        free(*ptr);
        free(*col);
        free(*val);
        *ptr = NULL;
        *col = NULL;
        *val = NULL;
        return HBICG_E_NOMEM;
    }
    unsigned e = 0;
    (*ptr)[0] = 0;
    for (unsigned i = 0; i < n; i++) {
        for (unsigned a = d->ptr[i]; a < d->ptr[i + 1]; a++) {
            (*col)[e] = d->col[a];
            (*val)[e++] = d->val[a];
        }
        for (unsigned a = o->ptr[i]; a < o->ptr[i + 1]; a++) {
            (*col)[e] = o->col[a];
            (*val)[e++] = o->val[a];
        }
        (*ptr)[i + 1] = e;
    }
    return HBICG_OK;
}

static int dropin(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                  double *r_loc, double *sigma, int sigma_len, int seed, int form, int use_graph) {
    if (A_info->cols != A_info->rows) {
        printf("Error: matrix is not square.\n");
        exit(1);
    }
    hbicg_params p;
    hbicg_params_default(&p);
    p.tol = g_tol;
    p.max_iter = g_maxit;
    p.switching = g_switching;
    p.form = form;
    p.use_graph = use_graph;
    p.refine = 0; /* the reference's entry points return the reference's x */
    const CSR_Matrix *A = A_loc_diag;
    unsigned *ptr = A->ptr, *col = A->col;
    double *val = A->val;
    int merged = 0;
    if (A_loc_offd && A_loc_offd->nz > 0 && A_loc_offd->ptr) {
        int rc = merged_csr(A_loc_diag, A_loc_offd, &ptr, &col, &val);
        if (rc) return -rc;
        merged = 1;
    }
    hbicg_stats st;
    memset(&st, 0, sizeof st);
    const unsigned nz = ptr[A->rows];
    int rc = hbicg_solve(A->rows, nz, ptr, col, val, r_loc, sigma, sigma_len, seed, &p, x_loc_set, r_loc, &st);
    if (merged) {
        free(ptr);
        free(col);
        free(val);
    }
    if (rc != HBICG_OK && rc != HBICG_E_MAXITER && rc != HBICG_E_BREAKDOWN) {
        fprintf(stderr, "hbicg: %s (%s)\n", hbicg_status_string(rc), hbicg_last_message());
        return -rc;
    }
    return st.k;
}

int shifted_lopbicg_dynamic(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                            double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_FUSED, 1);
}

int shifted_lopbicg_static(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_PLAIN, 0);
}

int shifted_lopbicg_normal(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_FUSED, 0);
}
