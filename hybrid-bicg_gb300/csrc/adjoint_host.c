/* Adjoint of a shifted family (config 5): gradients of
 *     J = sum_j w_j c^T x_j,   (A + sigma_j I) x_j = b
 * with respect to A's values, b and the shifts, from one forward family and
 * one transposed family (A^T + sigma_j I) y_j = c on the same shifts.
 *
 * The reference has no adjoint and no A^T path (its solver only moves
 * forward, src/solver_dynamic.c).  A^T is built on the GPU from A's CSR by
 * the stable COO -> CSR (columns become rows; entries of a new row keep the
 * order of their old rows), and the transposed family is an ordinary solve
 * with the reference's semantics, so it can be checked against the reference
 * solver run on A^T with right-hand side c. */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "host_internal.h"

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) {                                   \
            hbicg__set_message(cudaGetErrorString(e_));            \
            rc = HBICG_E_CUDA;                                     \
            goto done;                                             \
        }                                                          \
    } while (0)

int hbicg_matrix_transpose(hbicg_matrix *A, hbicg_matrix **At) {
    if (!A || !At) return HBICG_E_ARG;
    const hbk_matrix *k = hbicg__matrix_kernel_view(A);
    hbicg_context *ctx = hbicg__matrix_context(A);
    cudaStream_t st = (cudaStream_t)hbicg_context_stream(ctx);
    unsigned *rows = NULL;
    int rc = HBICG_OK;
    CK(cudaMalloc((void **)&rows, sizeof(unsigned) * ((size_t)k->nnz + 1)));
    CK((cudaError_t)hbk_entry_rows(k->n, k->ptr, rows, st));
    CK(cudaStreamSynchronize(st));
    /* (row, col) -> (col, row): the new rows are the old columns */
    rc = hbicg_matrix_from_coo(ctx, k->n, k->nnz, k->col, rows, k->val, HBICG_DEVICE, At);
done:
    cudaFree(rows);
    return rc;
}

int hbicg_adjoint_gradients(hbicg_matrix *A, int m, const double *X, unsigned long long ldx, const double *Lam,
                            unsigned long long ldl, const double *w, double *dJ_dval, double *dJ_db,
                            double *dJ_dsigma) {
    if (!A || m < 0) return HBICG_E_ARG;
    const hbk_matrix *k = hbicg__matrix_kernel_view(A);
    cudaStream_t st = (cudaStream_t)hbicg_context_stream(hbicg__matrix_context(A));
    unsigned *rows = NULL;
    void *tmp = NULL;
    int rc = HBICG_OK;
    if (dJ_dval) {
        CK(cudaMalloc((void **)&rows, sizeof(unsigned) * ((size_t)k->nnz + 1)));
        CK((cudaError_t)hbk_entry_rows(k->n, k->ptr, rows, st));
        CK((cudaError_t)hbk_grad_val(k->nnz, rows, k->col, m, X, ldx, Lam, ldl, w, dJ_dval, st));
    }
    if (dJ_db) CK((cudaError_t)hbk_grad_b(k->n, m, Lam, ldl, w, dJ_db, st));
    if (dJ_dsigma && m > 0) {
        CK(cudaMalloc(&tmp, hbk_adjoint_tmp_bytes(m)));
        CK((cudaError_t)hbk_shift_dots(k->n, m, X, ldx, Lam, ldl, 0, w, -1.0, dJ_dsigma, tmp, st));
    }
    CK(cudaStreamSynchronize(st));
done:
    cudaFree(rows);
    cudaFree(tmp);
    return rc;
}

int hbicg_adjoint(hbicg_matrix *A, hbicg_matrix *At, const double *b, const double *sigma, int m, int seed,
                  const double *w, const double *c, const hbicg_params *p, double *J, double *dJ_dval, double *dJ_db,
                  double *dJ_dsigma, double *x_out, hbicg_stats *fwd, hbicg_stats *adj) {
    if (!A || !b || !sigma || !c || m < 1) return HBICG_E_ARG;
    hbicg_context *ctx = hbicg__matrix_context(A);
    cudaStream_t st = (cudaStream_t)hbicg_context_stream(ctx);
    const hbk_matrix *k = hbicg__matrix_kernel_view(A);
    const size_t n = k->n;
    hbicg_matrix *T = At;
    hbicg_solver *s1 = NULL, *s2 = NULL;
    double *dX = NULL, *dY = NULL, *dw = NULL, *dc = NULL, *dcx = NULL, *ddv = NULL, *ddb = NULL, *dds = NULL;
    double *hcx = NULL;
    void *tmp = NULL;
    int rc = HBICG_OK, r1 = HBICG_OK, r2 = HBICG_OK;
    if (!T && (rc = hbicg_matrix_transpose(A, &T)) != HBICG_OK) return rc;
    CK(cudaMalloc((void **)&dX, sizeof(double) * n * (size_t)m));
    CK(cudaMalloc((void **)&dY, sizeof(double) * n * (size_t)m));
    CK(cudaMalloc((void **)&dw, sizeof(double) * (size_t)m));
    CK(cudaMalloc((void **)&dc, sizeof(double) * (n ? n : 1)));
    CK(cudaMalloc((void **)&dcx, sizeof(double) * (size_t)m));
    CK(cudaMalloc((void **)&dds, sizeof(double) * (size_t)m));
    CK(cudaMalloc((void **)&ddb, sizeof(double) * (n ? n : 1)));
    CK(cudaMalloc((void **)&ddv, sizeof(double) * ((size_t)k->nnz + 1)));
    CK(cudaMalloc(&tmp, hbk_adjoint_tmp_bytes(m)));
    if (w) CK(cudaMemcpy(dw, w, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dc, c, sizeof(double) * n, cudaMemcpyHostToDevice));
    /* forward family on A, transposed family on A^T (same shifts and seed) */
    if ((rc = hbicg_solver_create(ctx, A, m, p, &s1)) != HBICG_OK) goto done;
    r1 = hbicg_solver_run(s1, b, sigma, seed, HBICG_HOST, dX, NULL, HBICG_DEVICE, fwd);
    if (r1 != HBICG_OK && r1 != HBICG_E_MAXITER) {
        rc = r1;
        goto done;
    }
    if ((rc = hbicg_solver_create(ctx, T, m, p, &s2)) != HBICG_OK) goto done;
    r2 = hbicg_solver_run(s2, c, sigma, seed, HBICG_HOST, dY, NULL, HBICG_DEVICE, adj);
    if (r2 != HBICG_OK && r2 != HBICG_E_MAXITER) {
        rc = r2;
        goto done;
    }
    const double *pw = w ? dw : NULL;
    /* J = sum_j w_j c.x_j (per-shift dots summed on the host in shift order) */
    CK((cudaError_t)hbk_shift_dots((unsigned)n, m, dX, n, dc, 0, 1, pw, 1.0, dcx, tmp, st));
    if ((rc = hbicg_adjoint_gradients(A, m, dX, n, dY, n, pw, dJ_dval ? ddv : NULL, dJ_db ? ddb : NULL,
                                      dJ_dsigma ? dds : NULL)) != HBICG_OK)
        goto done;
    hcx = malloc(sizeof(double) * (size_t)m);
    if (!hcx) {
        rc = HBICG_E_NOMEM;
        goto done;
    }
    CK(cudaMemcpy(hcx, dcx, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
    if (J) {
        double s = 0.0;
        for (int j = 0; j < m; ++j) s += hcx[j];
        *J = s;
    }
    if (dJ_dval) CK(cudaMemcpy(dJ_dval, ddv, sizeof(double) * k->nnz, cudaMemcpyDeviceToHost));
    if (dJ_db) CK(cudaMemcpy(dJ_db, ddb, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (dJ_dsigma) CK(cudaMemcpy(dJ_dsigma, dds, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
    if (x_out) CK(cudaMemcpy(x_out, dX, sizeof(double) * n * (size_t)m, cudaMemcpyDeviceToHost));
    rc = r1 != HBICG_OK ? r1 : r2;
done:
    hbicg_solver_destroy(s1);
    hbicg_solver_destroy(s2);
    if (T && T != At) hbicg_matrix_destroy(T);
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dw);
    cudaFree(dc);
    cudaFree(dcx);
    cudaFree(ddv);
    cudaFree(ddb);
    cudaFree(dds);
    cudaFree(tmp);
    free(hcx);
    return rc;
}
