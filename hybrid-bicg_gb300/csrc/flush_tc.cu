// Basis flush on the tensor cores: x_j += xi_j Pmat_j + sum_l Xc[j][l] V[l],
// p_j = rho_j Pmat_j + sum_l Pc[j][l] V[l], with FP64 accuracy from BF16
// tcgen05 MMAs.
//
// GB300 runs FP64 at ~1.2 TFLOP/s, so the FP64 form of this product is the
// solver's bottleneck.  Here each FP64 operand is cut into nine signed 7-bit
// integer digits (63 bits) against a power-of-two scale — per output row for
// the coefficients, per vector element for the basis, after normalising every
// basis slot by a power of two — so that every digit is exact in BF16.  A
// digit product summed over K = 64 slots stays below 2^24 even when all pairs
// of one diagonal (s + t = d) are summed together, so each diagonal
// d = 0..8 accumulates exactly in its own FP32 TMEM accumulator.  Diagonals
// past 8 are dropped (their total is below 2^-53 of the row/element scale,
// the accuracy of an FP64 dot product of the same length).  The epilogue joins
// the nine exact diagonal sums in 128-bit integer arithmetic and rounds once
// to FP64; only the own-vector terms use the FP64 pipe.  (The digit splitting
// is the error-free splitting of Ozaki, Ogita, Oishi and Rump for matrix
// products, arranged here so that the exact sums fit TMEM.)
//
// One CTA per SM (205 KB of shared memory), persistent over tiles of 48
// vector elements; 128 output rows per group of 64 shifts (x rows, then p
// rows).  Per tile: build the basis digits in shared memory, one thread
// issues 45 x 4 MMAs (M=128, N=48, K=16) into nine accumulators, the warps
// read TMEM back and write x and p.  Every wait is bounded: a timeout sets an
// error flag, the CTA skips its remaining work and still frees its TMEM.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "hbk_device.cuh"

using namespace hbk;

namespace {

constexpr int TC_M = 128;
constexpr int TC_N = 48;
constexpr int TC_K = 64;
constexpr int NDIG = 9;
constexpr int NDIAG = 9;
constexpr int A_SLICE = TC_M * TC_K * 2;  // 16384 B
constexpr int B_SLICE = TC_N * TC_K * 2;  // 6144 B
constexpr int A_BYTES = NDIG * A_SLICE;   // 147456 B
constexpr int B_BYTES = NDIG * B_SLICE;   // 55296 B
constexpr int TC_THREADS = 256;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_MISC = 4096;
constexpr int SMEM_BYTES = A_BYTES + B_BYTES + SMEM_MISC;
constexpr long long WAIT_LIMIT = 1ll << 26;  // polls of an mbarrier before giving up
constexpr int EXP_NONE = -100000;            // exponent of an all-zero row or column

// byte offset of element (row, k) in a K-major, no-swizzle UMMA operand:
// core matrices of 8 rows x 16 bytes; K-adjacent core matrices 128 B apart
// (leading byte offset), 8-row groups 1024 B apart (stride byte offset).
__device__ __forceinline__ uint32_t umma_off(int row, int k) {
    return (uint32_t)(((row >> 3) * 8 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29),
// SBO >> 4 (32-45), fixed 0b001 (46-48), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try(bar, parity)) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// exponent e with |v| < 2^e for a nonzero double, from its bits
__device__ __forceinline__ int exp_of_bits(uint64_t bits) {
    const int eb = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & ((1ull << 52) - 1);
    if (eb) return eb - 1022;
    return (64 - __clzll((long long)frac)) - 1074;
}

// 63-bit magnitude of |v| * 2^(63 - scale) (truncated), v given by its bits
__device__ __forceinline__ uint64_t fixed63(uint64_t bits, int scale) {
    const int eb = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & ((1ull << 52) - 1);
    const uint64_t M = eb ? (frac | (1ull << 52)) : frac;
    const int e2 = (eb ? eb : 1) - 1075;
    const int sh = e2 + 63 - scale;
    if (M == 0 || sh <= -64) return 0;
    return sh >= 0 ? (M << sh) : (M >> (-sh));
}

// round-to-nearest FP64 of T * 2^k, T an exact 128-bit integer
__device__ __forceinline__ double i128_scaled(__int128 T, int k) {
    if (T == 0) return 0.0;
    const bool neg = T < 0;
    unsigned __int128 U = neg ? (unsigned __int128)(-T) : (unsigned __int128)T;
    const uint64_t hi = (uint64_t)(U >> 64), lo = (uint64_t)U;
    int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    uint64_t mant;
    if (p <= 52) {
        mant = (uint64_t)(U << (52 - p));
    } else {
        const int s = p - 52;
        const unsigned __int128 m = U >> s;
        const unsigned __int128 rem = U - (m << s);
        const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
        mant = (uint64_t)m;
        if (rem > half || (rem == half && (mant & 1))) {
            ++mant;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                ++p;
            }
        }
    }
    const int eb = p + k + 1023;
    if (eb >= 2047) return neg ? -INFINITY : INFINITY;
    if (eb <= 0) return neg ? -0.0 : 0.0;  // below the normal range: negligible here
    const uint64_t bits = ((uint64_t)neg << 63) | ((uint64_t)eb << 52) | (mant & ((1ull << 52) - 1));
    return __longlong_as_double((long long)bits);
}

// exact FP64 of v * 2^e for |v| < 2^53, built from bits (no FP64 instruction)
__device__ __forceinline__ double i64_scaled(long long v, int e) {
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    const uint64_t u = neg ? (uint64_t)(-v) : (uint64_t)v;
    const int p = 63 - __clzll((long long)u);
    const uint64_t mant = u << (52 - p);
    const int eb = p + e + 1023;
    if (eb >= 2047) return neg ? -INFINITY : INFINITY;
    if (eb <= 0) return neg ? -0.0 : 0.0;  // below the normal range: negligible here
    return __longlong_as_double((long long)(((uint64_t)neg << 63) | ((uint64_t)eb << 52) | (mant & ((1ull << 52) - 1))));
}

constexpr int SROW = TC_N + 1;  // staged row stride in doubles (avoids bank conflicts)

struct TcArgs {
    const double *V;      // basis [slots][ld]
    size_t ld;
    unsigned n;
    int L;                // slots in use (<= 64)
    const unsigned long long *slot_max;  // bits of max |V[l]| per slot
    const unsigned char *aimg;           // per group: 9 digit slices of the 128 x 64 coefficient block
    const int *rowexp;    // per group: [128]
    const double *rown;   // per group: [128] own-term scalar (xi for x rows, rho for p rows)
    double *X, *Pmat;     // [m][ld]
    int m, keep_p;
    int *err;
};

// ---- per-slot max |V[l]| (bits of a non-negative double order as integers)
__global__ void __launch_bounds__(NT) k_slot_max(const double *__restrict__ V, size_t ld, unsigned n, int L,
                                                 unsigned long long *slot_max) {
    const int l = blockIdx.y;
    if (l >= L) return;
    const double *v = V + (size_t)l * ld;
    unsigned long long mx = 0;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v[i]));
        mx = b > mx ? b : mx;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = t > mx ? t : mx;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(slot_max + l, mx);
}

// ---- coefficient digits: one block per output row, one thread per slot
__global__ void __launch_bounds__(TC_K) k_flush_prep(const double *__restrict__ Xc, const double *__restrict__ Pc,
                                                     int cap, const double *__restrict__ own, int m, int L,
                                                     const unsigned long long *__restrict__ slot_max,
                                                     unsigned char *aimg, int *rowexp, double *rown) {
    __shared__ unsigned long long s_max[2];
    const int r = blockIdx.x, g = blockIdx.y, l = threadIdx.x;
    const int which = r >> 6, j = g * 64 + (r & 63);
    double a = 0.0;
    if (j < m && l < L) {
        const double c = (which ? Pc : Xc)[(size_t)j * cap + l];
        const unsigned long long sm = slot_max[l];
        a = sm ? ldexp(c, exp_of_bits(sm)) : 0.0;  // fold the slot's scale into the coefficient
    }
    unsigned long long b = (unsigned long long)__double_as_longlong(fabs(a));
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
        b = t > b ? t : b;
    }
    if ((l & 31) == 0) s_max[l >> 5] = b;
    __syncthreads();
    const unsigned long long rmax = s_max[0] > s_max[1] ? s_max[0] : s_max[1];
    const int E = rmax ? exp_of_bits(rmax) : EXP_NONE;
    const uint64_t Q = rmax ? fixed63((uint64_t)__double_as_longlong(a), E) : 0;
    const bool neg = a < 0.0;
    unsigned char *img = aimg + (size_t)g * A_BYTES;
    const uint32_t off = umma_off(r, l);
#pragma unroll
    for (int s = 0; s < NDIG; ++s) {
        const int dgt = (int)((Q >> (56 - 7 * s)) & 127);
        const __nv_bfloat16 h = __float2bfloat16_rn((float)(neg ? -dgt : dgt));
        *reinterpret_cast<__nv_bfloat16 *>(img + (size_t)s * A_SLICE + off) = h;
    }
    if (l == 0) {
        rowexp[g * TC_M + r] = E;
        rown[g * TC_M + r] = (j < m) ? own[2 * (size_t)j + which] : 0.0;
    }
}

// ---- the tensor-core flush
__global__ void __launch_bounds__(TC_THREADS, 1) k_flush_tc(TcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;
    unsigned char *sB = smem + A_BYTES;
    unsigned char *misc = smem + A_BYTES + B_BYTES;
    uint64_t *bar_a = reinterpret_cast<uint64_t *>(misc);
    uint64_t *bar_mma = reinterpret_cast<uint64_t *>(misc + 8);
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(misc + 16);
    int *s_fail = reinterpret_cast<int *>(misc + 20);
    int *s_slotexp = reinterpret_cast<int *>(misc + 64);                // [64]
    int *s_colexp = reinterpret_cast<int *>(misc + 64 + 256);           // [4][48]
    int *s_rowexp = reinterpret_cast<int *>(misc + 64 + 256 + 768);     // [128]
    double *s_rown = reinterpret_cast<double *>(misc + 64 + 256 + 768 + 512);  // [128]

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = blockIdx.y;

    if (tid == 0) {
        mbar_init(bar_a, 1);
        mbar_init(bar_mma, 1);
        *s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid < TC_K) {
        const unsigned long long sm = tid < a.L ? a.slot_max[tid] : 0ull;
        s_slotexp[tid] = sm ? exp_of_bits(sm) : 0;
    }
    if (tid < TC_M) {
        s_rowexp[tid] = a.rowexp[g * TC_M + tid];
        s_rown[tid] = a.rown[g * TC_M + tid];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;

    // the coefficient digits of this group: one bulk copy per slice
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar_a)),
                     "r"((uint32_t)A_BYTES)
                     : "memory");
        const unsigned char *src = a.aimg + (size_t)g * A_BYTES;
        for (int s = 0; s < NDIG; ++s)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(sA + s * A_SLICE)),
                "l"(src + (size_t)s * A_SLICE), "r"((uint32_t)A_SLICE), "r"(smem_u32(bar_a))
                : "memory");
    }
    bool a_ok = mbar_wait(bar_a, 0);
    if (!a_ok) atomicExch(s_fail, 1);
    __syncthreads();

    const unsigned n = a.n;
    const unsigned ntiles = (n + TC_N - 1) / TC_N;
    const size_t ld = a.ld;
    uint32_t phase = 0;
    bool mma_pending = false;
    for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (*(volatile int *)s_fail) break;
        const unsigned i0 = t * TC_N;
        // ---- basis digits: thread (column i, quarter q) covers slots 16q..16q+15
        uint64_t vb[16];
        const int i = tid % TC_N, q = tid / TC_N;
        const bool builder = tid < 4 * TC_N;
        int emax = EXP_NONE;
        if (builder) {
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int l = 16 * q + u;
                double v = 0.0;
                if (l < a.L && i0 + i < n) v = a.V[(size_t)l * ld + i0 + i];
                vb[u] = (uint64_t)__double_as_longlong(v);
                if (v != 0.0) emax = max(emax, exp_of_bits(vb[u]) - s_slotexp[l]);
            }
            s_colexp[q * TC_N + i] = emax;
        }
        __syncthreads();
        if (builder) {
            int F = s_colexp[i];
            F = max(F, s_colexp[TC_N + i]);
            F = max(F, s_colexp[2 * TC_N + i]);
            F = max(F, s_colexp[3 * TC_N + i]);
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
                const int l = 16 * q + u;
                const uint64_t Q0 = vb[u] && F != EXP_NONE ? fixed63(vb[u], F + s_slotexp[l]) : 0;
                const uint64_t Q1 = vb[u + 1] && F != EXP_NONE ? fixed63(vb[u + 1], F + s_slotexp[l + 1]) : 0;
                const bool n0 = (int64_t)vb[u] < 0, n1 = (int64_t)vb[u + 1] < 0;
                const uint32_t off = umma_off(i, l);
#pragma unroll
                for (int s = 0; s < NDIG; ++s) {
                    const int d0 = (int)((Q0 >> (56 - 7 * s)) & 127), d1 = (int)((Q1 >> (56 - 7 * s)) & 127);
                    __nv_bfloat162 h;
                    h.x = __float2bfloat16_rn((float)(n0 ? -d0 : d0));
                    h.y = __float2bfloat16_rn((float)(n1 ? -d1 : d1));
                    *reinterpret_cast<__nv_bfloat162 *>(sB + s * B_SLICE + off) = h;
                }
            }
        }
        // digits written by threads must be visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (builder && q == 0) s_colexp[i] = max(max(s_colexp[i], s_colexp[TC_N + i]),
                                                 max(s_colexp[2 * TC_N + i], s_colexp[3 * TC_N + i]));

        // ---- MMAs: diagonal d into accumulator columns [48 d, 48 d + 48)
        if (tid == 0) {
            tc_fence_after();
            const uint64_t ad0 = umma_desc(smem_u32(sA)), bd0 = umma_desc(smem_u32(sB));
            for (int d = 0; d < NDIAG; ++d) {
                bool first = true;
                for (int s = max(0, d - (NDIG - 1)); s <= min(d, NDIG - 1); ++s) {
                    const int tt = d - s;
                    for (int kk = 0; kk < TC_K / 16; ++kk) {
                        // start-address field: (offset >> 4) adds without carry (smem < 256 KB)
                        const uint64_t ad = ad0 + (uint64_t)((s * A_SLICE + kk * 256) >> 4);
                        const uint64_t bd = bd0 + (uint64_t)((tt * B_SLICE + kk * 256) >> 4);
                        const uint32_t acc = first ? 0u : 1u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem + d * TC_N),
                            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                            : "memory");
                        first = false;
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(bar_mma))
                         : "memory");
        }
        if (!mbar_wait(bar_mma, phase)) {
            atomicExch(s_fail, 1);
            mma_pending = true;
        }
        phase ^= 1;
        tc_fence_after();
        __syncthreads();
        if (*(volatile int *)s_fail) break;

        // ---- epilogue.  The x and p tiles of the group (64 rows x 48 columns)
        // are staged in shared memory (the digit buffer is free once the MMAs
        // are done) with coalesced loads; warp w then reads TMEM lanes
        // 32 (w % 4) .. +31 (one output row per thread), columns 24 (w / 4) .. +23.
        double *sXo = reinterpret_cast<double *>(sB);
        double *sPo = sXo + 64 * SROW;
        const int jbase = g * 64;
        const int rows = min(64, a.m - jbase);
        for (int e = tid; e < 64 * TC_N; e += TC_THREADS) {
            const int jj = e / TC_N, cc = e % TC_N;
            const unsigned ii = i0 + cc;
            const bool in = jj < rows && ii < n;
            const size_t o = (size_t)(jbase + jj) * ld + ii;
            sXo[jj * SROW + cc] = in ? a.X[o] : 0.0;
            sPo[jj * SROW + cc] = (in && a.Pmat) ? a.Pmat[o] : 0.0;
        }
        __syncthreads();
        const int lq = warp & 3, ch = warp >> 2;
        const int r = 32 * lq + lane;
        const int which = r >> 6, jj = r & 63;
        const bool live = jj < rows && (which == 0 || a.keep_p);
        const int E = s_rowexp[r];
        const double own = s_rown[r];
        for (int c = 0; c < 3; ++c) {
            const int col0 = 24 * ch + 8 * c;
            uint32_t dv[NDIAG][8];
#pragma unroll
            for (int d = 0; d < NDIAG; ++d) {
                const uint32_t taddr = tmem + ((uint32_t)(32 * lq) << 16) + (uint32_t)(d * TC_N + col0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                    : "=r"(dv[d][0]), "=r"(dv[d][1]), "=r"(dv[d][2]), "=r"(dv[d][3]), "=r"(dv[d][4]), "=r"(dv[d][5]),
                      "=r"(dv[d][6]), "=r"(dv[d][7])
                    : "r"(taddr));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            double pn[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int cc = col0 + u;
                const int F = s_colexp[cc];
                double G = 0.0;
                if (E != EXP_NONE && F != EXP_NONE) {
                    // T = sum_d D_d 2^(7 (8 - d)) as hi * 2^35 + lo, both exact in int64
                    long long hi = __float2int_rz(__uint_as_float(dv[0][u]));
#pragma unroll
                    for (int d = 1; d < 4; ++d) hi = hi * 128 + __float2int_rz(__uint_as_float(dv[d][u]));
                    long long lo = __float2int_rz(__uint_as_float(dv[4][u]));
#pragma unroll
                    for (int d = 5; d < NDIAG; ++d) lo = lo * 128 + __float2int_rz(__uint_as_float(dv[d][u]));
                    const long long q = lo >> 35;            // floor(lo / 2^35)
                    const long long th = hi + q;             // T = th 2^35 + tl, 0 <= tl < 2^35
                    const long long tl = lo - q * (1ll << 35);
                    const int k = E + F - 70;
                    G = i64_scaled(th, k + 35) + i64_scaled(tl, k);  // one rounding
                }
                // x rows write now (they read the old p); p rows wait for the barrier
                if (live && which == 0) sXo[jj * SROW + cc] = fma(own, sPo[jj * SROW + cc], sXo[jj * SROW + cc]) + G;
                pn[u] = fma(own, sPo[jj * SROW + cc], G);
            }
            __syncthreads();
            if (live && which == 1) {
#pragma unroll
                for (int u = 0; u < 8; ++u) sPo[jj * SROW + col0 + u] = pn[u];
            }
        }
        __syncthreads();
        for (int e = tid; e < 64 * TC_N; e += TC_THREADS) {
            const int jr = e / TC_N, cc = e % TC_N;
            const unsigned ii = i0 + cc;
            if (jr < rows && ii < n) {
                const size_t o = (size_t)(jbase + jr) * ld + ii;
                a.X[o] = sXo[jr * SROW + cc];
                if (a.keep_p) a.Pmat[o] = sPo[jr * SROW + cc];
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    // every path ends here: let copies and MMAs still in flight after a
    // timeout finish (bounded), then free TMEM
    if (!a_ok) mbar_wait(bar_a, 0);
    if (mma_pending) mbar_wait(bar_mma, phase ^ 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    if (tid == 0 && *s_fail) atomicExch(a.err, 1);
}

}  // namespace

extern "C" {

size_t hbk_flush_tc_workspace_bytes(int m) {
    const int groups = (m + 63) / 64;
    return 256 + 64 * sizeof(unsigned long long) + (size_t)groups * (A_BYTES + TC_M * (sizeof(int) + sizeof(double)));
}

int hbk_flush_tc_max_slots(void) { return TC_K; }

// x_j (and p_j when keep_p) from the first L basis slots on the tensor cores;
// ws: device workspace of hbk_flush_tc_workspace_bytes(m), err: device int.
int hbk_flush_tc_run(const double *V, size_t ld, unsigned n, int L, const double *Xc, const double *Pc, int cap,
                     const double *own, int m, double *X, double *Pmat, int keep_p, void *ws, int *err,
                     cudaStream_t st) {
    if (L > TC_K || L < 1 || m < 1 || n == 0) return (int)cudaErrorInvalidValue;
    const int groups = (m + 63) / 64;
    unsigned char *w = (unsigned char *)ws;
    unsigned long long *slot_max = (unsigned long long *)(w + 256);
    unsigned char *aimg = w + 256 + 64 * sizeof(unsigned long long);
    int *rowexp = (int *)(aimg + (size_t)groups * A_BYTES);
    double *rown = (double *)(rowexp + groups * TC_M);
    cudaError_t e = cudaMemsetAsync(slot_max, 0, 64 * sizeof(unsigned long long), st);
    if (e) return (int)e;
    dim3 gs(grid_for(n, 16) < 64 ? grid_for(n, 16) : 64, L);
    k_slot_max<<<gs, NT, 0, st>>>(V, ld, n, L, slot_max);
    k_flush_prep<<<dim3(TC_M, groups), TC_K, 0, st>>>(Xc, Pc, cap, own, m, L, slot_max, aimg, rowexp, rown);
    static int attr_set = 0;
    if (!attr_set) {
        e = cudaFuncSetAttribute(k_flush_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e) return (int)e;
        attr_set = 1;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned ntiles = (n + TC_N - 1) / TC_N;
    const unsigned gx = ntiles < (unsigned)sms ? ntiles : (unsigned)sms;
    TcArgs args{V, ld, n, L, slot_max, aimg, rowexp, rown, X, Pmat, m, keep_p, err};
    k_flush_tc<<<dim3(gx, groups), TC_THREADS, SMEM_BYTES, st>>>(args);
    return (int)cudaGetLastError();
}

}  // extern "C"
