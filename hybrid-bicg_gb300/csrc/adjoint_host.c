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
#include <pthread.h>
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

/* A^T built into context `into` (its arrays, its format work on that
 * context's stream) */
static int transpose_into(hbicg_matrix *A, hbicg_context *into, hbicg_matrix **At) {
    const hbk_matrix *k = hbicg__matrix_kernel_view(A);
    cudaStream_t st = (cudaStream_t)hbicg_context_stream(hbicg__matrix_context(A));
    unsigned *rows = NULL;
    int rc = HBICG_OK;
    CK(hbicg__dev_alloc((void **)&rows, sizeof(unsigned) * ((size_t)k->nnz + 1), st));
    CK((cudaError_t)hbk_entry_rows(k->n, k->ptr, rows, st));
    CK(cudaStreamSynchronize(st));
    /* (row, col) -> (col, row): the new rows are the old columns */
    rc = hbicg_matrix_from_coo(into, k->n, k->nnz, k->col, rows, k->val, HBICG_DEVICE, At);
    cudaStreamSynchronize((cudaStream_t)hbicg_context_stream(into)); /* done reading rows */
done:
    hbicg__dev_free(rows, st);
    cudaStreamSynchronize(st);
    return rc;
}

int hbicg_matrix_transpose(hbicg_matrix *A, hbicg_matrix **At) {
    if (!A || !At) return HBICG_E_ARG;
    return transpose_into(A, hbicg__matrix_context(A), At);
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
        CK(hbicg__dev_alloc((void **)&rows, sizeof(unsigned) * ((size_t)k->nnz + 1), st));
        CK((cudaError_t)hbk_entry_rows(k->n, k->ptr, rows, st));
        CK((cudaError_t)hbk_grad_val(k->nnz, rows, k->col, m, X, ldx, Lam, ldl, w, dJ_dval, st));
    }
    if (dJ_db) CK((cudaError_t)hbk_grad_b(k->n, m, Lam, ldl, w, dJ_db, st));
    if (dJ_dsigma && m > 0) {
        CK(hbicg__dev_alloc(&tmp, hbk_adjoint_tmp_bytes(m), st));
        CK((cudaError_t)hbk_shift_dots(k->n, m, X, ldx, Lam, ldl, 0, w, -1.0, dJ_dsigma, tmp, st));
    }
    CK(cudaStreamSynchronize(st));
done:
    hbicg__dev_free(rows, st);
    hbicg__dev_free(tmp, st);
    cudaStreamSynchronize(st);
    return rc;
}

/* one family solved into device memory on the matrix's own context.  When the
 * two matrices live on different contexts (streams), the transposed family
 * runs on a second host thread while the forward family runs on the
 * caller's: the solves are independent, and each leaves gaps on the GPU
 * (between its short kernels, around its host round trips) that the other
 * fills.  Results do not depend on the overlap: every grid and reduction
 * order is fixed by the matrix and the device, not by what else runs. */
typedef struct {
    hbicg_matrix *M;
    const hbicg_params *p;
    const double *rhs, *sigma;
    double *X;
    hbicg_stats *st;
    int m, seed, device, rc;
    char msg[256];
} famrun_t;

static void *famrun(void *arg) {
    famrun_t *f = arg;
    hbicg_solver *s = NULL;
    hbicg_context *ctx = hbicg__matrix_context(f->M);
    if (cudaSetDevice(f->device) != cudaSuccess) {
        f->rc = HBICG_E_CUDA;
        strncpy(f->msg, "cudaSetDevice failed on the transposed family's thread", sizeof f->msg - 1);
        return NULL;
    }
    f->rc = hbicg_solver_create(ctx, f->M, f->m, f->p, &s);
    if (f->rc == HBICG_OK) f->rc = hbicg_solver_run(s, f->rhs, f->sigma, f->seed, HBICG_HOST, f->X, NULL, HBICG_DEVICE, f->st);
    hbicg_solver_destroy(s);
    cudaStreamSynchronize((cudaStream_t)hbicg_context_stream(ctx));
    if (f->rc != HBICG_OK) strncpy(f->msg, hbicg_last_message(), sizeof f->msg - 1);
    return NULL;
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
    hbicg_context *ctx2 = NULL;
    double *dX = NULL, *dY = NULL, *dw = NULL, *dc = NULL, *dcx = NULL, *ddv = NULL, *ddb = NULL, *dds = NULL;
    double *hcx = NULL;
    void *tmp = NULL;
    int rc = HBICG_OK, r1 = HBICG_OK, r2 = HBICG_OK, dev = 0;
    if (!T) {
        /* A^T on a second context of its own, so that the two families can run at once */
        if ((rc = hbicg_context_create(&ctx2)) != HBICG_OK) return rc;
        if ((rc = transpose_into(A, ctx2, &T)) != HBICG_OK) {
            hbicg_context_destroy(ctx2);
            return rc;
        }
    }
    /* device buffers from the library's pool (no cudaMalloc/cudaFree mapping per call) */
    CK(hbicg__dev_alloc((void **)&dX, sizeof(double) * n * (size_t)m, st));
    CK(hbicg__dev_alloc((void **)&dY, sizeof(double) * n * (size_t)m, st));
    CK(hbicg__dev_alloc((void **)&dw, sizeof(double) * (size_t)m, st));
    CK(hbicg__dev_alloc((void **)&dc, sizeof(double) * (n ? n : 1), st));
    CK(hbicg__dev_alloc((void **)&dcx, sizeof(double) * (size_t)m, st));
    CK(hbicg__dev_alloc((void **)&dds, sizeof(double) * (size_t)m, st));
    CK(hbicg__dev_alloc((void **)&ddb, sizeof(double) * (n ? n : 1), st));
    CK(hbicg__dev_alloc((void **)&ddv, sizeof(double) * ((size_t)k->nnz + 1), st));
    CK(hbicg__dev_alloc(&tmp, hbk_adjoint_tmp_bytes(m), st));
    if (w) CK(cudaMemcpyAsync(dw, w, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dc, c, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetDevice(&dev));
    /* forward family on A, transposed family on A^T (same shifts and seed):
     * at the same time when A^T has a stream of its own, else one after the other */
    {
        famrun_t fa = {A, p, b, sigma, dX, fwd, m, seed, dev, HBICG_OK, {0}};
        famrun_t fb = {T, p, c, sigma, dY, adj, m, seed, dev, HBICG_OK, {0}};
        pthread_t th;
        const int threaded = hbicg__matrix_context(T) != ctx && pthread_create(&th, NULL, famrun, &fb) == 0;
        famrun(&fa);
        if (threaded) pthread_join(th, NULL);
        else famrun(&fb);
        r1 = fa.rc;
        r2 = fb.rc;
        if (r1 != HBICG_OK && r1 != HBICG_E_MAXITER) {
            hbicg__set_message(fa.msg);
            rc = r1;
            goto done;
        }
        if (r2 != HBICG_OK && r2 != HBICG_E_MAXITER) {
            hbicg__set_message(fb.msg);
            rc = r2;
            goto done;
        }
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
    cudaStreamSynchronize(st);
    if (T && T != At) hbicg_matrix_destroy(T);
    if (ctx2) hbicg_context_destroy(ctx2);
    hbicg__dev_free(dX, st);
    hbicg__dev_free(dY, st);
    hbicg__dev_free(dw, st);
    hbicg__dev_free(dc, st);
    hbicg__dev_free(dcx, st);
    hbicg__dev_free(ddv, st);
    hbicg__dev_free(ddb, st);
    hbicg__dev_free(dds, st);
    hbicg__dev_free(tmp, st);
    cudaStreamSynchronize(st);
    free(hcx);
    return rc;
}
