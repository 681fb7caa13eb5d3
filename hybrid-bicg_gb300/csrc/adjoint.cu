// Gradient kernels of the adjoint of a shifted family.
//
// For J = sum_j w_j c^T x_j with (A + sigma_j I) x_j = b, and the adjoint
// solutions y_j of (A^T + sigma_j I) y_j = c (lambda_j = w_j y_j):
//   dJ/db        = sum_j lambda_j
//   dJ/dsigma_j  = -lambda_j . x_j
//   dJ/dA[i][k]  = -sum_j lambda_j[i] x_j[k]   (on A's pattern: one value per entry)
// The same kernels serve any upstream gradient: given X and Lambda (lambda_j
// solving (A^T + sigma_j I) lambda_j = g_j), they return the gradients with
// respect to the values, b and the shifts.  The reference has no adjoint; the
// formulas are the standard ones for a linear solve.  Dot products are
// deterministic (fixed per-block partials summed in order).
#include "hbk_device.cuh"

using namespace hbk;

namespace {

constexpr int DOT_GRID = 512;  // partial sums per shift

__global__ void __launch_bounds__(NT) k_entry_rows(unsigned n, const unsigned *__restrict__ ptr, unsigned *rows) {
    for (size_t r = blockIdx.x * (size_t)NT + threadIdx.x; r < n; r += (size_t)gridDim.x * NT)
        for (unsigned e = ptr[r]; e < ptr[r + 1]; ++e) rows[e] = (unsigned)r;
}

// part[j * DOT_GRID + b] = sum over block b's elements of a_j . x_j, where
// a_j = A[j] (a_shared: one vector for all j)
__global__ void __launch_bounds__(NT) k_shift_dots(unsigned n, const double *__restrict__ X, size_t ldx,
                                                   const double *__restrict__ Aa, size_t lda, int a_shared,
                                                   double *part) {
    __shared__ double red[NW];
    const int j = blockIdx.y;
    const double *x = X + (size_t)j * ldx;
    const double *a = Aa + (a_shared ? 0 : (size_t)j * lda);
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) acc = fma(a[i], x[i], acc);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = acc;
}

// out[j] = scale * w_j * sum_b part[j][b] (in block order)
__global__ void k_sum_parts(int m, int g, const double *__restrict__ part, const double *__restrict__ w, double scale,
                            double *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    double s = 0.0;
    for (int b = 0; b < g; ++b) s += part[(size_t)j * g + b];
    out[j] = scale * (w ? w[j] : 1.0) * s;
}

// db[i] = sum_j w_j Y[j][i]
__global__ void __launch_bounds__(NT) k_grad_b(unsigned n, int m, const double *__restrict__ Y, size_t ldy,
                                               const double *__restrict__ w, double *db) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) {
        double s = 0.0;
        for (int j = 0; j < m; ++j) s = fma(w ? w[j] : 1.0, Y[(size_t)j * ldy + i], s);
        db[i] = s;
    }
}

// dval[e] = -sum_j w_j Y[j][row(e)] X[j][col(e)]
__global__ void __launch_bounds__(NT) k_grad_val(unsigned nnz, const unsigned *__restrict__ rows,
                                                 const unsigned *__restrict__ col, int m, const double *__restrict__ X,
                                                 size_t ldx, const double *__restrict__ Y, size_t ldy,
                                                 const double *__restrict__ w, double *dval) {
    for (size_t e = blockIdx.x * (size_t)NT + threadIdx.x; e < nnz; e += (size_t)gridDim.x * NT) {
        const unsigned i = rows[e], k = col[e];
        double s = 0.0;
        for (int j = 0; j < m; ++j)
            s = fma((w ? w[j] : 1.0) * Y[(size_t)j * ldy + i], X[(size_t)j * ldx + k], s);
        dval[e] = -s;
    }
}

}  // namespace

extern "C" {

int hbk_entry_rows(unsigned n, const unsigned *ptr, unsigned *rows, cudaStream_t st) {
    k_entry_rows<<<grid_for(n ? n : 1, 4), NT, 0, st>>>(n, ptr, rows);
    return (int)cudaGetLastError();
}

size_t hbk_adjoint_tmp_bytes(int m) { return sizeof(double) * (size_t)(m > 0 ? m : 1) * DOT_GRID; }

// out[j] = scale * w_j * (a_j . x_j); device pointers; tmp of hbk_adjoint_tmp_bytes(m)
int hbk_shift_dots(unsigned n, int m, const double *X, size_t ldx, const double *a, size_t lda, int a_shared,
                   const double *w, double scale, double *out, void *tmp, cudaStream_t st) {
    if (m <= 0) return 0;
    k_shift_dots<<<dim3(DOT_GRID, m), NT, 0, st>>>(n, X, ldx, a, lda, a_shared, (double *)tmp);
    k_sum_parts<<<(m + 63) / 64, 64, 0, st>>>(m, DOT_GRID, (const double *)tmp, w, scale, out);
    return (int)cudaGetLastError();
}

int hbk_grad_b(unsigned n, int m, const double *Y, size_t ldy, const double *w, double *db, cudaStream_t st) {
    k_grad_b<<<grid_for(n ? n : 1, 2), NT, 0, st>>>(n, m, Y, ldy, w, db);
    return (int)cudaGetLastError();
}

int hbk_grad_val(unsigned nnz, const unsigned *rows, const unsigned *col, int m, const double *X, size_t ldx,
                 const double *Y, size_t ldy, const double *w, double *dval, cudaStream_t st) {
    k_grad_val<<<grid_for(nnz ? nnz : 1, 2), NT, 0, st>>>(nnz, rows, col, m, X, ldx, Y, ldy, w, dval);
    return (int)cudaGetLastError();
}

}  // extern "C"
