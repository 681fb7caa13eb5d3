// True-residual norms without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they want to check a
// solve: code that runs while another component owns the device memory budget
// (a framework whose caching allocator has reserved the GPU), latency-bound
// loops that must not take cudaMalloc's implicit device synchronisation, or
// host callbacks that may not make allocating CUDA calls.  This entry point
// computes ||b - (A + sigma_j I) x_j|| / ||b|| for up to
// HBICG_NOALLOC_MAX_SHIFTS shifts with the same reduction kernels the solver
// uses for its own residual check, but takes its scratch (per-block partial
// sums, the last-block tickets and the squared norms) from one file-scope
// __device__ array instead of the allocator.
//
// The array is part of the library's device image: every GPU that loads the
// library holds it (about 1 MiB) until the process exits.  All calls share it,
// so calls whose kernels overlap on the GPU (other streams, other host
// threads) race on it; serialise them.  The first call on a device looks up
// the array's device address with cudaGetSymbolAddress (under a lock, once per
// device) and keeps it; make that first call before any stream capture.  The
// kept address belongs to the device's primary context: after
// cudaDeviceReset on that device the process must not call this entry point
// again.
#include <math.h>
#include <mutex>
#include <string.h>

#include "hbicg.h"
#include "hbk_device.cuh"

using namespace hbk;

namespace {

constexpr int kMaxShifts = HBICG_NOALLOC_MAX_SHIFTS;
// Blocks of the residual products and of the b.b dot, whatever the device:
// both launches are capped at this many blocks, one partial sum each.
constexpr int kMaxGrid = 2048;
constexpr size_t kPartials = (size_t)(kMaxShifts + 1) * kMaxGrid;  // doubles
constexpr size_t kSums = kMaxShifts + 8;                           // doubles
constexpr size_t kTickets = kMaxShifts + 16;                       // unsigned
constexpr size_t kBytes = (kPartials + kSums) * sizeof(double) + kTickets * sizeof(unsigned);

// Host code must never pass this symbol to a kernel: on the host it names a
// stand-in, not device memory.  Its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kBytes];

constexpr int kMaxDevices = 64;
static void *g_scratch_dev[kMaxDevices];
static std::mutex g_scratch_lock;

__global__ void k_norms(const double *sq, const double *bb, int m, double *res) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) res[j] = sqrt(sq[j]) / sqrt(*bb);
}

}  // namespace

extern "C" const hbk_matrix *hbicg__matrix_kernel_view(const hbicg_matrix *A);
extern "C" void hbicg__set_message(const char *msg);

extern "C" int hbicg_true_residuals_noalloc(hbicg_matrix *A, const double *x, unsigned long long ldx, const double *b,
                                            const double *sigma, int m, double *res, void *stream) {
    if (!A || (m > 0 && (!x || !b || !sigma || !res))) {
        hbicg__set_message("hbicg_true_residuals_noalloc: null argument");
        return HBICG_E_ARG;
    }
    if (m < 0 || m > kMaxShifts) {
        hbicg__set_message("hbicg_true_residuals_noalloc: m must be in [0, HBICG_NOALLOC_MAX_SHIFTS] (64)");
        return HBICG_E_ARG;
    }
    const hbk_matrix *K = hbicg__matrix_kernel_view(A);
    if (m == 0 || K->n == 0) return HBICG_OK;
    if (ldx < K->n) {
        hbicg__set_message("hbicg_true_residuals_noalloc: ldx smaller than the number of rows");
        return HBICG_E_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        hbicg__set_message("hbicg_true_residuals_noalloc: no usable current device");
        return HBICG_E_CUDA;
    }
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_scratch_lock);
        if (!g_scratch_dev[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess || !p) {
                hbicg__set_message(cudaGetErrorString(e));
                return HBICG_E_CUDA;
            }
            g_scratch_dev[dev] = p;
        }
        base = g_scratch_dev[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    double *partials = (double *)base;
    double *sums = partials + kPartials;
    unsigned *tickets = (unsigned *)(sums + kSums);
    // the last-block tickets must start at zero (an earlier call that failed
    // part-way could have left one raised)
    if (cudaMemsetAsync(tickets, 0, kTickets * sizeof(unsigned), st) != cudaSuccess) {
        hbicg__set_message("hbicg_true_residuals_noalloc: clearing the tickets failed");
        return HBICG_E_CUDA;
    }
    int e = hbk_true_residuals_ld(K, x, (size_t)ldx, b, sigma, m, kMaxGrid, partials, tickets, sums, st);
    if (!e)
        e = hbk_dot_capped(K->n, b, b, kMaxGrid, partials + (size_t)kMaxShifts * kMaxGrid, tickets + kMaxShifts,
                           sums + kMaxShifts, st);
    if (!e) {
        k_norms<<<(m + 63) / 64, 64, 0, st>>>(sums, sums + kMaxShifts, m, res);
        e = (int)cudaGetLastError();
    }
    if (e) {
        hbicg__set_message(cudaGetErrorString((cudaError_t)e));
        return HBICG_E_CUDA;
    }
    return HBICG_OK;
}
