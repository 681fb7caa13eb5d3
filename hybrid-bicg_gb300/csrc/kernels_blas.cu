// Plain per-step kernels (one launch per step of the reference's iteration)
// and the CSR SpMV entry points.  The plain solver form drives these from the
// host exactly in the reference's order (src/solver_dynamic.c:156-256).
#include <stdio.h>

#include "hbk_device.cuh"

using namespace hbk;

namespace {

__global__ void __launch_bounds__(NT) k_copy(unsigned n, const double *__restrict__ x, double *__restrict__ y) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) y[i] = x[i];
}

__global__ void __launch_bounds__(NT) k_fill(unsigned n, double v, double *__restrict__ x) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) x[i] = v;
}

// y[i] += a * x[i]   (my_openmp_daxpy, src/openmp_vector.c:3-9)
__global__ void __launch_bounds__(NT) k_axpy(unsigned n, double a, const double *__restrict__ x,
                                             double *__restrict__ y) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) y[i] = fma(a, x[i], y[i]);
}

__global__ void __launch_bounds__(NT) k_scal(unsigned n, double a, double *__restrict__ x) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) x[i] *= a;
}

__global__ void __launch_bounds__(NT) k_dot(unsigned n, const double *__restrict__ x, const double *__restrict__ y,
                                            double *partials, unsigned *counter, double *out) {
    __shared__ double sh[NW];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) acc = fma(x[i], y[i], acc);
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    if (take_ticket(counter)) {
        double t = sum_partials(partials, gridDim.x, sh);
        if (threadIdx.x == 0) {
            *out = t;
            *counter = 0;
        }
    }
}

struct EpiStore {
    double *y;
    const double *x;
    double sigma;
    int add;
    __device__ void operator()(unsigned r, double acc) const { y[r] = add ? fma(sigma, x[r], acc) : acc; }
};

struct EpiAccum {
    double *y;
    __device__ void operator()(unsigned r, double acc) const { y[r] += acc; }
};

template <int FMT>
__global__ void __launch_bounds__(NT) k_spmv(hbk_matrix A, const double *__restrict__ x, double *__restrict__ y,
                                             double sigma, int add) {
    EpiStore epi{y, x, sigma, add};
    spmv_rows<FMT>(A, x, epi);
}

template <int FMT>
__global__ void __launch_bounds__(NT) k_spmv_acc(hbk_matrix A, const double *__restrict__ x, double *__restrict__ y) {
    EpiAccum epi{y};
    spmv_rows<FMT>(A, x, epi);
}

// out[j] = ||b - (A + sigma_j I) x_j||^2 ; one launch per shift block (grid.y = shift)
template <int FMT>
__device__ __forceinline__ void true_res_body(const hbk_matrix &A, const double *__restrict__ X, size_t ld,
                                              const double *__restrict__ b, const double *__restrict__ sigma,
                                              double *partials, unsigned *counters, double *out) {
    __shared__ double sh[NW];
    const int j = blockIdx.y;
    const double *xj = X + (size_t)j * ld;
    const double sg = sigma[j];
    double acc = 0.0;
    auto epi = [&](unsigned r, double ax) {
        const double res = b[r] - fma(sg, xj[r], ax);
        acc = fma(res, res, acc);
    };
    spmv_rows<FMT>(A, xj, epi);
    acc = block_sum(acc, sh);
    double *pj = partials + (size_t)j * gridDim.x;
    if (threadIdx.x == 0) pj[blockIdx.x] = acc;
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(counters + j, 1u) == gridDim.x - 1);
    __syncthreads();
    if (s_last) {
        __threadfence();
        double t = sum_partials(pj, gridDim.x, sh);
        if (threadIdx.x == 0) {
            out[j] = t;
            counters[j] = 0;
        }
    }
}

template <int FMT>
__global__ void __launch_bounds__(NT) k_true_res(hbk_matrix A, const double *__restrict__ X, size_t ld,
                                                 const double *__restrict__ b, const double *__restrict__ sigma,
                                                 double *partials, unsigned *counters, double *out) {
    true_res_body<FMT>(A, X, ld, b, sigma, partials, counters, out);
}
template <>
__global__ void __launch_bounds__(NT, HBK_HYB_MINB) k_true_res<HBK_FMT_HYB>(
    hbk_matrix A, const double *__restrict__ X, size_t ld, const double *__restrict__ b,
    const double *__restrict__ sigma, double *partials, unsigned *counters, double *out) {
    true_res_body<HBK_FMT_HYB>(A, X, ld, b, sigma, partials, counters, out);
}

// SELL-32 build: slice widths, then one thread per row writes its entries
// (column-major within the slice) and its padding (value 0, column = row).
// HYB slices from CSR: lane l of slice s copies row srow[32 s + l]; padding
// entries get value 0 and a column index of 0 (an empty lane's entries too)
__global__ void __launch_bounds__(NT) k_hyb_fill(unsigned nslice, const unsigned *__restrict__ srow, unsigned n,
                                                 const unsigned *__restrict__ ptr, const unsigned *__restrict__ col,
                                                 const double *__restrict__ val,
                                                 const unsigned long long *__restrict__ sptr,
                                                 double *__restrict__ sval, unsigned *__restrict__ scol) {
    const size_t tot = (size_t)nslice * 32;
    for (size_t t = blockIdx.x * (size_t)NT + threadIdx.x; t < tot; t += (size_t)gridDim.x * NT) {
        const size_t s = t >> 5;
        const unsigned lane = (unsigned)(t & 31);
        const unsigned long long base = sptr[s];
        const unsigned w = (unsigned)((sptr[s + 1] - base) >> 5);
        const unsigned r = srow[t];
        const unsigned a = r < n ? ptr[r] : 0, len = r < n ? ptr[r + 1] - ptr[r] : 0;
        for (unsigned e = 0; e < w; ++e) {
            const size_t o = base + 32 * (size_t)e + lane;
            sval[o] = e < len ? val[a + e] : 0.0;
            scol[o] = e < len ? col[a + e] : 0u;
        }
    }
}

// position of each row's first stored diagonal entry in the SELL-32 arrays
__global__ void __launch_bounds__(NT) k_sell_diag(unsigned n, const unsigned *__restrict__ ptr,
                                                  const unsigned long long *__restrict__ sptr,
                                                  const unsigned *__restrict__ scol,
                                                  unsigned long long *__restrict__ sdiag, int *missing) {
    for (unsigned r = blockIdx.x * NT + threadIdx.x; r < n; r += gridDim.x * NT) {
        const unsigned long long base = sptr[r >> 5] + (r & 31);
        const unsigned len = ptr[r + 1] - ptr[r];
        unsigned long long at = ~0ull;
        for (unsigned e = 0; e < len; ++e)
            if (scol[base + 32ull * e] == r) {
                at = base + 32ull * e;
                break;
            }
        sdiag[r] = at;
        if (at == ~0ull) *missing = 1;
    }
}

// sval_shift[sdiag[r]] = sval[sdiag[r]] + sigma (the rest copied before)
__global__ void __launch_bounds__(NT) k_fold_diag(unsigned n, const double *__restrict__ sval,
                                                  const unsigned long long *__restrict__ sdiag,
                                                  const double *__restrict__ sigma, double *__restrict__ sval_shift) {
    const double sg = *sigma;
    for (unsigned r = blockIdx.x * NT + threadIdx.x; r < n; r += gridDim.x * NT) {
        const unsigned long long d = sdiag[r];
        sval_shift[d] = sval[d] + sg;
    }
}

__global__ void __launch_bounds__(NT) k_sell_widths(unsigned n, const unsigned *__restrict__ ptr,
                                                    unsigned *__restrict__ w) {
    const unsigned ns = (n + 31) / 32;
    for (unsigned s = blockIdx.x * NT + threadIdx.x; s < ns; s += gridDim.x * NT) {
        unsigned mx = 0;
        const unsigned r1 = min(n, 32 * s + 32);
        for (unsigned r = 32 * s; r < r1; ++r) mx = max(mx, ptr[r + 1] - ptr[r]);
        w[s] = mx;
    }
}

__global__ void __launch_bounds__(NT) k_sell_fill(unsigned n, const unsigned *__restrict__ ptr,
                                                  const unsigned *__restrict__ col, const double *__restrict__ val,
                                                  const unsigned long long *__restrict__ sptr,
                                                  double *__restrict__ sval, unsigned *__restrict__ scol) {
    const unsigned n32 = (n + 31) / 32 * 32;
    for (unsigned r = blockIdx.x * NT + threadIdx.x; r < n32; r += gridDim.x * NT) {
        const unsigned s = r >> 5, lane = r & 31;
        const unsigned long long base = sptr[s];
        const unsigned w = (unsigned)((sptr[s + 1] - base) >> 5);
        const unsigned a = r < n ? ptr[r] : 0, len = r < n ? ptr[r + 1] - ptr[r] : 0;
        const unsigned self = r < n ? r : 0;
        for (unsigned e = 0; e < w; ++e) {
            const size_t o = base + 32 * (size_t)e + lane;
            sval[o] = e < len ? val[a + e] : 0.0;
            scol[o] = e < len ? col[a + e] : self;
        }
    }
}

}  // namespace

extern "C" {

int hbk_hyb_fill(unsigned nslice, const unsigned *srow, unsigned n, const unsigned *ptr, const unsigned *col,
                 const double *val, const unsigned long long *sptr, double *sval, unsigned *scol, cudaStream_t st) {
    if (!nslice) return 0;
    k_hyb_fill<<<grid_for(nslice * 32u, 1), NT, 0, st>>>(nslice, srow, n, ptr, col, val, sptr, sval, scol);
    return (int)cudaGetLastError();
}

int hbk_sell_diag(unsigned n, const unsigned *ptr, const unsigned long long *sptr, const unsigned *scol,
                  unsigned long long *sdiag, int *missing, cudaStream_t st) {
    if (!n) return 0;
    k_sell_diag<<<grid_for(n, 2), NT, 0, st>>>(n, ptr, sptr, scol, sdiag, missing);
    return (int)cudaGetLastError();
}

int hbk_fold_diag(unsigned n, const double *sval, unsigned long long len, const unsigned long long *sdiag,
                  const double *sigma, double *sval_shift, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(sval_shift, sval, sizeof(double) * len, cudaMemcpyDeviceToDevice, st);
    if (e || !n) return (int)e;
    k_fold_diag<<<grid_for(n, 2), NT, 0, st>>>(n, sval, sdiag, sigma, sval_shift);
    return (int)cudaGetLastError();
}

int hbk_sell_widths(unsigned n, const unsigned *ptr, unsigned *w, cudaStream_t st) {
    if (!n) return 0;
    k_sell_widths<<<grid_for((n + 31) / 32, 1), NT, 0, st>>>(n, ptr, w);
    return (int)cudaGetLastError();
}

int hbk_sell_fill(unsigned n, const unsigned *ptr, const unsigned *col, const double *val,
                  const unsigned long long *sptr, double *sval, unsigned *scol, cudaStream_t st) {
    if (!n) return 0;
    k_sell_fill<<<grid_for(n, 1), NT, 0, st>>>(n, ptr, col, val, sptr, sval, scol);
    return (int)cudaGetLastError();
}

int hbk_last_error(void) { return (int)cudaGetLastError(); }
const char *hbk_error_string(int code) { return cudaGetErrorString((cudaError_t)code); }

int hbk_device_sm_count(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

int hbk_copy(unsigned n, const double *x, double *y, cudaStream_t st) {
    if (!n) return 0;
    k_copy<<<grid_for(n, 4), NT, 0, st>>>(n, x, y);
    return (int)cudaGetLastError();
}

int hbk_fill(unsigned n, double v, double *x, cudaStream_t st) {
    if (!n) return 0;
    k_fill<<<grid_for(n, 4), NT, 0, st>>>(n, v, x);
    return (int)cudaGetLastError();
}

int hbk_zero(unsigned n, double *x, cudaStream_t st) { return hbk_fill(n, 0.0, x, st); }

int hbk_axpy(unsigned n, double a, const double *x, double *y, cudaStream_t st) {
    if (!n) return 0;
    k_axpy<<<grid_for(n, 4), NT, 0, st>>>(n, a, x, y);
    return (int)cudaGetLastError();
}

int hbk_scal(unsigned n, double a, double *x, cudaStream_t st) {
    if (!n) return 0;
    k_scal<<<grid_for(n, 4), NT, 0, st>>>(n, a, x);
    return (int)cudaGetLastError();
}

int hbk_dot(unsigned n, const double *x, const double *y, double *partials, unsigned *counter, double *out,
            cudaStream_t st) {
    k_dot<<<grid_for(n, 4), NT, 0, st>>>(n, x, y, partials, counter, out);
    return (int)cudaGetLastError();
}

int hbk_dot_capped(unsigned n, const double *x, const double *y, int grid_cap, double *partials, unsigned *counter,
                   double *out, cudaStream_t st) {
    int g = grid_for(n, 4);
    if (grid_cap >= 1 && g > grid_cap) g = grid_cap;
    k_dot<<<g, NT, 0, st>>>(n, x, y, partials, counter, out);
    return (int)cudaGetLastError();
}

int hbk_spmv_grid(unsigned nblk) {
    int g = grid_for(nblk * (unsigned)NT, 1);
    return g < 1 ? 1 : g;
}

int hbk_hyb_wave_blas(void) {
    int g = wave_grid<k_spmv<HBK_FMT_HYB>>(HBK_MAX_GRID);
    const int a = wave_grid<k_spmv_acc<HBK_FMT_HYB>>(HBK_MAX_GRID), t = wave_grid<k_true_res<HBK_FMT_HYB>>(HBK_MAX_GRID);
    if (a < g) g = a;
    return t < g ? t : g;
}

// MERGE form: one wave of the product kernel (its units are dealt round-robin,
// so a second wave would wait for whole CTAs of the first)
int hbk_merge_grid(unsigned units) {
    const int w = wave_grid<k_spmv<HBK_FMT_MERGE>>(HBK_MAX_GRID);
    const unsigned need = (units + NW - 1) / NW;  // a unit per warp
    const int g = need < (unsigned)w ? (int)need : w;
    return g < 1 ? 1 : g;
}

int hbk_spmv(const hbk_matrix *A, const double *x, double *y, double sigma, int sigma_add, cudaStream_t st) {
    if (!A->n) return 0;
    HBK_LAUNCH_FMT(*A, k_spmv, A->grid, NT, st, *A, x, y, sigma, sigma_add);
    return (int)cudaGetLastError();
}

int hbk_spmv_accumulate(const hbk_matrix *A, const double *x, double *y, cudaStream_t st) {
    if (!A->n) return 0;
    HBK_LAUNCH_FMT(*A, k_spmv_acc, A->grid, NT, st, *A, x, y);
    return (int)cudaGetLastError();
}

int hbk_true_residuals(const hbk_matrix *A, const double *X, const double *b, const double *sigma, int m,
                       double *partials, unsigned *counters, double *out, cudaStream_t st) {
    if (!A->n || m <= 0) return 0;
    size_t ld = ((size_t)A->n + 31) / 32 * 32;
    dim3 grid(A->grid, m);
    HBK_LAUNCH_FMT(*A, k_true_res, grid, NT, st, *A, X, ld, b, sigma, partials, counters, out);
    return (int)cudaGetLastError();
}

int hbk_true_residuals_ld(const hbk_matrix *A, const double *X, size_t ldx, const double *b, const double *sigma,
                          int m, int grid_cap, double *partials, unsigned *counters, double *out, cudaStream_t st) {
    if (!A->n || m <= 0) return 0;
    const int g = A->grid < grid_cap ? A->grid : grid_cap;
    dim3 grid(g, m);
    HBK_LAUNCH_FMT(*A, k_true_res, grid, NT, st, *A, X, ldx, b, sigma, partials, counters, out);
    return (int)cudaGetLastError();
}

// Row blocks: consecutive short rows are packed while the block stays within
// NT rows and HBK_TILE_NNZ nonzeros; a row longer than HBK_TILE_NNZ / 8 gets a
// block of its own and is reduced by the whole CTA.
unsigned hbk_plan_rows(unsigned n, const unsigned *ptr, unsigned *blk_row, unsigned char *blk_kind) {
    const unsigned long_row = HBK_TILE_NNZ / 8;
    unsigned nb = 0, i = 0;
    while (i < n) {
        const unsigned len = ptr[i + 1] - ptr[i];
        if (len > long_row) {
            if (blk_row) {
                blk_row[nb] = i;
                blk_kind[nb] = HBK_BLK_LONG;
            }
            nb++;
            i++;
            continue;
        }
        unsigned j = i, nz = 0;
        while (j < n && j - i < (unsigned)NT) {
            const unsigned l = ptr[j + 1] - ptr[j];
            if (l > long_row || nz + l > HBK_TILE_NNZ) break;
            nz += l;
            j++;
        }
        if (blk_row) {
            blk_row[nb] = i;
            blk_kind[nb] = HBK_BLK_TILE;
        }
        nb++;
        i = j;
    }
    if (blk_row) blk_row[nb] = n;
    return nb;
}

}  // extern "C"
