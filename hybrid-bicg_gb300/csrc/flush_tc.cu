// Basis flush on the tensor cores: x_j += xi_j Pmat_j + sum_l Xc[j][l] V[l],
// p_j = rho_j Pmat_j + sum_l Pc[j][l] V[l], with FP64 accuracy from BF16
// tcgen05 MMAs.
//
// GB300 runs FP64 at ~1.2 TFLOP/s, so the FP64 form of this product is the
// solver's bottleneck.  Here each FP64 operand becomes a signed 62-bit fixed
// point integer against a power-of-two scale — per output row for the
// coefficients, per vector element for the basis, after normalising every
// basis slot by a power of two — cut into nine balanced 7-bit digits in
// [-64, 64], each exact in BF16.  A digit product is at most 2^12, so the sum
// over K = 64 slots of all pairs of one diagonal (s + t = d, at most nine
// pairs) stays below 2^22: each diagonal d = 0..8 accumulates exactly in its
// own FP32 TMEM accumulator and converts to an integer with one FP32 add.
// Diagonals past 8 are dropped (their total is below 2^-54 of the
// row/element scale, the accuracy of an FP64 dot product of the same length).
// The epilogue joins the nine exact diagonal sums in 64-bit integer arithmetic
// (keeping floor(T / 2^12) of the 75-bit sum T: the dropped bits are below
// 2^-56 of the row x element scale) and rounds once to FP64; only the
// own-vector terms use the FP64 pipe.  (The digit splitting is the error-free
// splitting of Ozaki, Ogita, Oishi and Rump for matrix products, arranged here
// so that the exact sums fit TMEM.)
//
// One CTA per SM (226 KB of shared memory, all 512 TMEM columns), persistent
// over tiles of 48 vector elements (one panel of the panel-major x_j and p_j
// arrays, whose values for all shifts lie in one contiguous block); 128
// output rows per group of 64 shifts, ordered so that
// TMEM lanes 32q..32q+15 hold the x rows of shifts 16q..16q+15 and lanes
// 32q+16..32q+31 their p rows.  Warps 0-2 make the basis digits of a tile
// into one of two buffers (tile t+1's while the tensor core reads tile t's);
// one thread of warp 3 issues its MMAs (M=128, N up to 256, K=16; 52 per
// tile; coefficient digit slices 0-1 from TMEM, 2-8 from shared memory) into
// nine accumulators, so that the digit builders never wait behind the MMA
// issue; warps 4-15 empty the accumulators into registers first, so that the
// next tile's MMAs run while they round, add the own-vector terms and write x
// and p.  Every wait is bounded: a timeout sets an error flag, the CTA skips
// its remaining work and still frees its TMEM.
//
// Only the live shifts are formed: a shift that had converged by the previous
// flush has zero coefficients and own terms (0, 1) since that flush's reset,
// so its rows would come out unchanged.  The rows of a group are the live
// shifts in index order; a group without live shifts does nothing, and the
// epilogue warps of a TMEM quadrant without live rows sit the tiles out.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "hbk_device.cuh"

using namespace hbk;

namespace {

constexpr int TC_M = 128;
constexpr int TC_N = 48;
constexpr int TC_K = 64;
static_assert(TC_N == HBK_PANEL, "a tile is one panel of x_j and p_j");
constexpr int NDIG = 9;
constexpr int NDIAG = 9;
constexpr int A_SLICE = TC_M * TC_K * 2;  // 16384 B
constexpr int B_SLICE = TC_N * TC_K * 2;  // 6144 B
constexpr int A_BYTES = NDIG * A_SLICE;   // 147456 B (a group's coefficient digits in global memory)
constexpr int B_BYTES = NDIG * B_SLICE;   // 55296 B (one buffer of a tile's basis digits)
// Coefficient digit slices 0 and 1 live in TMEM (columns after the nine
// accumulators), the other seven in shared memory: that leaves room for two
// basis-digit buffers, so the builders write tile t+1's digits while the
// tensor core works through tile t.
constexpr int A_TMEM_SLICES = 2;
constexpr int A_SMEM_BYTES = (NDIG - A_TMEM_SLICES) * A_SLICE;  // 114688 B
constexpr int A_TCOL = NDIAG * TC_N;                             // first TMEM column of slice 0 (32 per slice)
constexpr int NBUF = 2;                                          // basis-digit buffers
constexpr int BUILD_WARPS = 3;            // warps 0-2: basis digits
constexpr int MMA_WARP = 3;               // warp 3: coefficient copy + MMA issue (one thread)
constexpr int EPI_WARP0 = MMA_WARP + 1;   // first epilogue warp (a multiple of 4: warp w reads TMEM quadrant w % 4)
constexpr int EPI_WARPS = 12;             // warps 4-15: epilogue
constexpr int TC_THREADS = 32 * (BUILD_WARPS + 1 + EPI_WARPS);
constexpr int BUILD_THREADS = 32 * BUILD_WARPS;
constexpr int EPI_COLS = TC_N / (EPI_WARPS / 4);  // 16 columns per epilogue thread
constexpr int ITEMS = (TC_K / 8) * TC_N;          // (slot octet, element) pairs per tile
constexpr int ITEMS_PER = ITEMS / BUILD_THREADS;  // 4
constexpr int TMEM_COLS = 512;
constexpr int SMEM_MISC = 6144;
constexpr int SMEM_BYTES = A_SMEM_BYTES + NBUF * B_BYTES + SMEM_MISC;  // 231424 B
constexpr long long WAIT_LIMIT = 1ll << 26;  // polls of an mbarrier before giving up
constexpr int EXP_NONE = -100000;            // exponent of an all-zero row or column
// sum_s 64 * 2^(56 - 7 s): adding it to a 62-bit signed value makes every
// 7-bit field of the sum the balanced digit + 64
constexpr uint64_t DIGIT_BIAS = 0x4081020408102040ull;
// magic FP32 1.5 * 2^23: for |D| < 2^22, bits(D + MAGIC) = MAGIC_BITS + D
constexpr float MAGIC = 12582912.0f;
constexpr uint32_t MAGIC_BITS = 0x4B400000u;
constexpr uint64_t HI_BIAS = (uint64_t)MAGIC_BITS * 2113665ull;  // * (2^21 + 2^14 + 2^7 + 1)
constexpr uint64_t MID_BIAS = (uint64_t)MAGIC_BITS * 66052ull;   // * (2^16 + 2^9 + 2^2)
constexpr uint64_t T_BIAS = (HI_BIAS << 23) + MID_BIAS;          // (mod 2^64)

static_assert(ITEMS % BUILD_THREADS == 0, "builder items");
static_assert(EPI_WARP0 % 4 == 0 && EPI_WARP0 + EPI_WARPS == TC_THREADS / 32, "epilogue warps: whole quadrant sets");
static_assert((TC_THREADS / 32 - 1 - EPI_WARP0) / 4 == EPI_WARPS / 4 - 1, "epilogue column groups");
static_assert(EPI_COLS % 4 == 0 && TC_N % 8 == 0, "epilogue columns");
static_assert(A_TCOL + 32 * A_TMEM_SLICES <= TMEM_COLS, "accumulators and the TMEM coefficient slices fit TMEM");
static_assert(SMEM_BYTES <= 232448, "shared memory of one CTA");
static_assert(A_SMEM_BYTES % 1024 == 0 && B_BYTES % 1024 == 0, "1024-byte aligned operand buffers");

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

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
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

// bounded wait; false on timeout or when another warp has already failed
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, const int *fail) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try(bar, parity)) return true;
        if (i > 64) {
            if ((i & 1023) == 0 && *(const volatile int *)fail) return false;
            __nanosleep(64);
        }
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

// v * 2^(62 - scale) truncated toward zero, as a two's complement integer
// (|v| < 2^scale, so the result is below 2^62), plus DIGIT_BIAS.  The
// significand M < 2^53 is placed at M 2^10 and shifted right by
// r = 1023 + scale - max(eb, 1) >= 0 (|v| < 2^scale bounds the left shift
// M 2^(62 - scale + eb - 1075) by 2^10).
__device__ __forceinline__ uint64_t biased62(uint64_t bits, int scale) {
    const int eb = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & ((1ull << 52) - 1);
    const uint64_t M = eb ? (frac | (1ull << 52)) : frac;
    const int r = 1023 + scale - (eb ? eb : 1);
    uint64_t q = r < 64 ? (M << 10) >> r : 0;
    const uint64_t sg = (uint64_t)((int64_t)bits >> 63);  // 0 or all ones
    q = (q ^ sg) - sg;
    return q + DIGIT_BIAS;
}

// balanced digit s (weight 2^(56 - 7 s)) of a biased value, as an exact float
template <int S>
__device__ __forceinline__ float digit(uint64_t U) {
    const uint32_t e = S == 0 ? (uint32_t)(U >> 56) : ((uint32_t)(U >> (56 - 7 * S)) & 127u);
    return __uint_as_float(0x4B000000u | e) - 8388672.0f;  // (2^23 + e) - (2^23 + 64)
}

template <int S>
__device__ __forceinline__ uint32_t digit_pair(uint64_t U0, uint64_t U1) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(digit<S>(U0), digit<S>(U1));
    return *reinterpret_cast<const uint32_t *>(&h);
}

// 8 consecutive slots of one element (Us[0..7]) -> one 16-byte row of a core
// matrix in every digit slice
template <int S>
__device__ __forceinline__ void store_digits(unsigned char *sB, uint32_t off, const uint64_t *Us) {
    uint4 w;
    w.x = digit_pair<S>(Us[0], Us[1]);
    w.y = digit_pair<S>(Us[2], Us[3]);
    w.z = digit_pair<S>(Us[4], Us[5]);
    w.w = digit_pair<S>(Us[6], Us[7]);
    *reinterpret_cast<uint4 *>(sB + S * B_SLICE + off) = w;
    if constexpr (S + 1 < NDIG) store_digits<S + 1>(sB, off, Us);
}

// 32 x 32 + 64 -> 64-bit multiply-add
__device__ __forceinline__ uint64_t madw(uint32_t a, uint32_t b, uint64_t c) {
    uint64_t d;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// floor(T / 2^12) of the exact diagonal sum T = sum_d D_d 2^(7 (8 - d)), from
// the biased FP32 bits B_d = MAGIC_BITS + D_d.  |D_d| <= (d + 1) 64 2^12, so
// |T| < 2^74.03 and the result fits a signed 64-bit integer; the dropped bits
// are below 2^-56 of the row x element scale (the dropped diagonals: 2^-54).
// Arithmetic is modulo 2^64 (the biases cancel exactly).
__device__ __forceinline__ long long diag_sum(const uint32_t (&B)[NDIAG]) {
    const uint64_t h = madw(B[0], 1u << 21, madw(B[1], 1u << 14, madw(B[2], 1u << 7, (uint64_t)B[3])));
    const uint64_t mid = madw(B[4], 1u << 16, madw(B[5], 1u << 9, (uint64_t)B[6] << 2));
    const int lo = (int)(B[7] * 128u + B[8] - MAGIC_BITS * 129u);  // D_7 2^7 + D_8, |.| < 2^29
    return (long long)((h << 23) + mid - T_BIAS + (uint64_t)(long long)(lo >> 12));
}

// T 2^k rounded to FP64: round half up on the 64-bit magnitude, whose leading
// bit is normalised to bit 63 (error <= 0.5 ulp of the result)
__device__ __forceinline__ double join_t(long long T, int k) {
    const long long sg = T >> 63;
    const unsigned long long a = (unsigned long long)((T ^ sg) - sg);
    if (a == 0) return 0.0;
    const int z = __clzll((long long)a);
    const unsigned long long W = a << z;
    const unsigned long long mant = (W >> 11) + ((W >> 10) & 1);  // 2^52 .. 2^53 (carries into the exponent)
    const int ebm1 = 63 - z + k + 1022;                             // biased exponent - 1
    if ((unsigned)ebm1 > 2044u) {
        if (ebm1 < 0) return sg ? -0.0 : 0.0;  // below the normal range: negligible here
        return sg ? -INFINITY : INFINITY;
    }
    const unsigned long long bits = ((unsigned long long)ebm1 << 52) + mant;
    return __longlong_as_double((long long)(bits | ((unsigned long long)sg << 63)));
}

// one 32-byte sector per lane and instruction (x and p rows are read and
// written 4 doubles at a time; 16-byte pieces of a sector written by separate
// instructions cost partial-sector traffic)
__device__ __forceinline__ void ld_sector(const double *p, double &a, double &b, double &c, double &d) {
    asm volatile("ld.global.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(a), "=d"(b), "=d"(c), "=d"(d) : "l"(p));
}
__device__ __forceinline__ void st_sector(double *p, double a, double b, double c, double d) {
    asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}

struct TcArgs {
    const double *V;      // basis [slots][ld]
    size_t ld;
    unsigned n;
    int L;                // slots in use (<= 64)
    const unsigned long long *slot_max;  // bits of max |V[l]| per slot
    const unsigned char *aimg;           // per group: 9 digit slices of the 128 x 64 coefficient block
    const int *rowexp;    // per group: [128]
    const double *rown;   // per group: [128] own-term scalar (xi for x rows, rho for p rows)
    double *X, *Pmat;     // panel-major, m systems
    int m, keep_p;
    const int *live;      // [0]: number of live shifts; [1 ..]: their indices, ascending
    int *err;
};

// live shifts: not converged (conv_k == 0) or converged after iteration
// k_last (the last one the previous flush covered); one warp, index order
__global__ void k_flush_live(const int *__restrict__ conv_k, int m, int k_last, int *live) {
    int cnt = 0;
    for (int base = 0; base < m; base += 32) {
        const int j = base + (int)threadIdx.x;
        bool on = false;
        if (j < m) {
            int c = conv_k ? conv_k[j] : 0;
            c = c < 0 ? -c : c;  // a shift that broke down at k stopped there like a converged one
            on = c == 0 || c > k_last;
        }
        const unsigned b = __ballot_sync(0xffffffffu, on);
        if (on) live[1 + cnt + __popc(b & ((1u << threadIdx.x) - 1u))] = j;
        cnt += __popc(b);
    }
    if (threadIdx.x == 0) live[0] = cnt;
}

// ---- per-slot max |V[l]| (bits of a non-negative double order as integers)
__global__ void __launch_bounds__(NT) k_slot_max(const double *__restrict__ V, size_t ld, unsigned n, int L,
                                                 unsigned long long *slot_max) {
    const int l = blockIdx.y;
    if (l >= L) return;
    const double *v = V + (size_t)l * ld;
    unsigned long long mx = 0;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v[i]) & 0x7FFFFFFFFFFFFFFFull;
        mx = b > mx ? b : mx;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = t > mx ? t : mx;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(slot_max + l, mx);
}

// slot maxima from the partial maxima kept by the kernels that wrote the slots
// (one warp per slot)
__global__ void k_fold_slot_max(const unsigned long long *__restrict__ part, int L, unsigned long long *slot_max) {
    const int l = blockIdx.x;
    if (l >= L) return;
    unsigned long long m = part[(size_t)l * HBK_SLOT_SPREAD + threadIdx.x];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if (threadIdx.x == 0) slot_max[l] = m;
}

// TMEM lane / A row r of a group -> (x or p, shift within the group)
__device__ __forceinline__ int row_which(int r) { return (r >> 4) & 1; }
__device__ __forceinline__ int row_shift(int r) { return ((r >> 5) << 4) | (r & 15); }

// ---- coefficient digits: one block per output row, one thread per slot
__global__ void __launch_bounds__(TC_K) k_flush_prep(const double *__restrict__ Xc, const double *__restrict__ Pc,
                                                     int cap, const double *__restrict__ own, int L,
                                                     const unsigned long long *__restrict__ slot_max,
                                                     const int *__restrict__ live, unsigned char *aimg, int *rowexp,
                                                     double *rown) {
    __shared__ unsigned long long s_max[2];
    const int r = blockIdx.x, g = blockIdx.y, l = threadIdx.x;
    const int which = row_which(r), pos = g * 64 + row_shift(r);
    if (g * 64 >= live[0]) return;  // the whole group is idle
    const int j = pos < live[0] ? live[1 + pos] : -1;
    double a = 0.0;
    if (j >= 0 && l < L) {
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
    const uint64_t U = (rmax && a != 0.0) ? biased62((uint64_t)__double_as_longlong(a), E) : DIGIT_BIAS;
    unsigned char *img = aimg + (size_t)g * A_BYTES;
    const uint32_t off = umma_off(r, l);
    const float d[NDIG] = {digit<0>(U), digit<1>(U), digit<2>(U), digit<3>(U), digit<4>(U),
                           digit<5>(U), digit<6>(U), digit<7>(U), digit<8>(U)};
#pragma unroll
    for (int s = 0; s < NDIG; ++s)
        *reinterpret_cast<__nv_bfloat16 *>(img + (size_t)s * A_SLICE + off) = __float2bfloat16_rn(d[s]);
    if (l == 0) {
        rowexp[g * TC_M + r] = E;
        rown[g * TC_M + r] = (j >= 0) ? own[2 * (size_t)j + which] : 0.0;
    }
}

// ---- the tensor-core flush
__global__ void __launch_bounds__(TC_THREADS, 1) k_flush_tc(TcArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;                 // coefficient digit slices 2 .. 8
    unsigned char *sB = smem + A_SMEM_BYTES;  // NBUF basis-digit buffers, tile it in buffer it % 2
    unsigned char *misc = smem + A_SMEM_BYTES + NBUF * B_BYTES;
    // Tiles alternate between the two basis-digit buffers, and the barriers
    // that hand a buffer between the builders and the tensor core come in
    // pairs (one per buffer): a parity wait is only sound while the waiter is
    // at most one phase behind, and the builders now run two tiles ahead.
    uint64_t *bar_a = reinterpret_cast<uint64_t *>(misc);           // coefficient digits landed
    uint64_t *bar_full = reinterpret_cast<uint64_t *>(misc + 8);     // [2] basis digits of a tile written
    uint64_t *bar_mma = reinterpret_cast<uint64_t *>(misc + 24);     // [2] MMAs of a tile done
    uint64_t *bar_ready = reinterpret_cast<uint64_t *>(misc + 40);   // MMAs issued (orders s_F for the epilogue)
    uint64_t *bar_tfree = reinterpret_cast<uint64_t *>(misc + 48);   // accumulators read out
    uint64_t *bar_cexp = reinterpret_cast<uint64_t *>(misc + 56);    // builders' partial exponents written
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(misc + 64);
    int *s_fail = reinterpret_cast<int *>(misc + 68);
    int *s_slotexp = reinterpret_cast<int *>(misc + 128);            // [64]
    int *s_cexp = reinterpret_cast<int *>(misc + 384);               // [2][8][48] per slot octet
    int *s_F = reinterpret_cast<int *>(misc + 3456);                 // [4][48] element exponents, ring
    int *s_rowexp = reinterpret_cast<int *>(misc + 4224);            // [128]
    double *s_rown = reinterpret_cast<double *>(misc + 4736);        // [128], ends at 5760

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = blockIdx.y;
    // live rows of this group; the whole CTA leaves (before any barrier or
    // TMEM allocation) when there are none
    const int n_live = a.live[0];
    const int g_live = n_live - 64 * g;
    if (g_live <= 0) return;
    const int live_quads = g_live >= 64 ? 4 : (g_live + 15) / 16;  // TMEM quadrants with a live row

    if (tid == 0) {
        mbar_init(bar_a, 1);
        mbar_init(bar_full, BUILD_THREADS);
        mbar_init(bar_full + 1, BUILD_THREADS);
        mbar_init(bar_mma, 1);
        mbar_init(bar_mma + 1, 1);
        mbar_init(bar_ready, 1);
        mbar_init(bar_tfree, (EPI_WARPS / 4) * live_quads);
        mbar_init(bar_cexp, BUILD_THREADS);
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
    // coefficient digit slices 0 and 1 into TMEM: lane r holds row r, each
    // 32-bit column two consecutive k (the lower k in the low half), slice s
    // at columns A_TCOL + 32 s ..  Warps 4-7 each write their own quadrant.
    if (warp >= EPI_WARP0 && warp < EPI_WARP0 + 4) {
        const int r = 32 * (warp & 3) + lane;
        const unsigned char *src = a.aimg + (size_t)g * A_BYTES;
#pragma unroll
        for (int s = 0; s < A_TMEM_SLICES; ++s) {
            uint32_t col[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const uint32_t lo = *reinterpret_cast<const unsigned short *>(src + s * A_SLICE + umma_off(r, 2 * c));
                const uint32_t hi = *reinterpret_cast<const unsigned short *>(src + s * A_SLICE + umma_off(r, 2 * c + 1));
                col[c] = lo | (hi << 16);
            }
            const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(A_TCOL + 32 * s);
            asm volatile(
                "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
                "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
                "r"(col[0]), "r"(col[1]), "r"(col[2]), "r"(col[3]), "r"(col[4]), "r"(col[5]), "r"(col[6]),
                "r"(col[7]), "r"(col[8]), "r"(col[9]), "r"(col[10]), "r"(col[11]), "r"(col[12]), "r"(col[13]),
                "r"(col[14]), "r"(col[15]), "r"(col[16]), "r"(col[17]), "r"(col[18]), "r"(col[19]), "r"(col[20]),
                "r"(col[21]), "r"(col[22]), "r"(col[23]), "r"(col[24]), "r"(col[25]), "r"(col[26]), "r"(col[27]),
                "r"(col[28]), "r"(col[29]), "r"(col[30]), "r"(col[31])
                : "memory");
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    const unsigned n = a.n;
    const unsigned ntiles = (n + TC_N - 1) / TC_N;
    const size_t ld = a.ld;
    bool a_ok = true;
    int issued = 0;  // the MMA thread: MMA batches committed

    if (warp < BUILD_WARPS) {
        // ---- builders: the basis digits of every tile.  They never issue
        // MMAs, so their work for the next tile (loads, exponents) runs while
        // the tensor core works through the current one.
        // item (octet o, element i): slots 8o..8o+7 of element i0 + i
        int io[ITEMS_PER], ii[ITEMS_PER];
#pragma unroll
        for (int u = 0; u < ITEMS_PER; ++u) {
            const int it = tid + BUILD_THREADS * u;
            io[u] = it / TC_N;
            ii[u] = it % TC_N;
        }
        double v[ITEMS_PER][8];
        auto load_tile = [&](unsigned t) {
            const unsigned i0 = t * TC_N;
#pragma unroll
            for (int u = 0; u < ITEMS_PER; ++u)
#pragma unroll
                for (int w = 0; w < 8; ++w) {
                    const int l = 8 * io[u] + w;
                    v[u][w] = (l < a.L && i0 + ii[u] < n) ? __ldcs(a.V + (size_t)l * ld + i0 + ii[u]) : 0.0;
                }
        };
        int it = 0;
        if (blockIdx.x < ntiles) load_tile(blockIdx.x);
        for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
            if (*(volatile int *)s_fail) break;
            // phase A (overlaps the previous tile's MMAs): element exponents;
            // s_cexp alternates between two buffers
            int *cexp = s_cexp + (it & 1) * ITEMS;
            int em[ITEMS_PER];
#pragma unroll
            for (int u = 0; u < ITEMS_PER; ++u) {
                int e = EXP_NONE;
#pragma unroll
                for (int w = 0; w < 8; ++w) {
                    // |v| < 2^(eb - 1022) for every v, zero and subnormals included
                    const int eb = (int)((uint64_t)__double_as_longlong(v[u][w]) >> 52) & 0x7ff;
                    e = max(e, eb - 1022 - s_slotexp[8 * io[u] + w]);
                }
                em[u] = e;
                cexp[io[u] * TC_N + ii[u]] = e;
            }
            // (an mbarrier, not a named barrier: a builder that gave up must not hang the others)
            mbar_arrive(bar_cexp);
            if (!mbar_wait(bar_cexp, it & 1, s_fail)) {
                atomicExch(s_fail, 1);
                break;
            }
            int Fv[ITEMS_PER];
#pragma unroll
            for (int u = 0; u < ITEMS_PER; ++u) {
                int F = em[u];
#pragma unroll
                for (int o = 0; o < TC_K / 8; ++o) F = max(F, cexp[o * TC_N + ii[u]]);
                Fv[u] = F;
            }
            // phase B: this tile's digit buffer is free once the MMAs of the
            // tile before the previous one (the same buffer) are done
            if (it >= NBUF && !mbar_wait(bar_mma + (it & 1), ((it >> 1) - 1) & 1, s_fail)) {
                atomicExch(s_fail, 1);
                break;
            }
            unsigned char *sBt = sB + (it & 1) * B_BYTES;
#pragma unroll
            for (int u = 0; u < ITEMS_PER; ++u) {
                uint64_t U[8];
#pragma unroll
                for (int w = 0; w < 8; ++w)
                    U[w] = biased62((uint64_t)__double_as_longlong(v[u][w]), Fv[u] + s_slotexp[8 * io[u] + w]);
                if (io[u] == 0) s_F[(it & 3) * TC_N + ii[u]] = Fv[u];
                store_digits<0>(sBt, umma_off(ii[u], 8 * io[u]), U);
            }
            // digits written by threads must be visible to the tensor core (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(bar_full + (it & 1));
            // the next tile's basis values are in flight during this tile's MMAs
            if (t + gridDim.x < ntiles) load_tile(t + gridDim.x);
        }
    } else if (warp == MMA_WARP) {
        // ---- one thread loads the coefficient digits and issues every MMA
        if (lane == 0) {
            // the coefficient digits of this group: one bulk copy per slice
            // the coefficient digit slices kept in shared memory (2 .. 8)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar_a)),
                         "r"((uint32_t)A_SMEM_BYTES)
                         : "memory");
            const unsigned char *src = a.aimg + (size_t)g * A_BYTES;
            for (int s = A_TMEM_SLICES; s < NDIG; ++s)
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(sA + (s - A_TMEM_SLICES) * A_SLICE)),
                    "l"(src + (size_t)s * A_SLICE), "r"((uint32_t)A_SLICE), "r"(smem_u32(bar_a))
                    : "memory");
            a_ok = mbar_wait(bar_a, 0, s_fail);
            if (!a_ok) atomicExch(s_fail, 1);
            const uint64_t ad0 = umma_desc(smem_u32(sA));
            int it = 0;
            for (unsigned t = blockIdx.x; t < ntiles && a_ok; t += gridDim.x, ++it) {
                const uint64_t bd0 = umma_desc(smem_u32(sB + (it & 1) * B_BYTES));
                bool ok = mbar_wait(bar_full + (it & 1), (it >> 1) & 1, s_fail);
                // the previous tile's accumulators must have been read out
                if (ok && it > 0) ok = mbar_wait(bar_tfree, (it - 1) & 1, s_fail);
                if (!ok) {
                    atomicExch(s_fail, 1);
                    break;
                }
                tc_fence_after();
                // diagonal d accumulates in columns [48 d, 48 d + 48).  The basis
                // digit slices lie one after another along N, so one MMA of
                // coefficient slice s against basis rows 0 .. 48 (9 - s) - 1,
                // written from column 48 s on, adds A_s B_t to diagonal s + t
                // for every t <= 8 - s (in two MMAs where N would pass 256).
#pragma unroll
                for (int kk = 0; kk < TC_K / 16; ++kk) {
#pragma unroll
                    for (int s = 0; s < NDIG; ++s) {
                        const int ntot = TC_N * (NDIG - s);
#pragma unroll
                        for (int part = 0; part * 256 < ntot; ++part) {
                            const int nn = ntot - part * 256 < 256 ? ntot - part * 256 : 256;
                            // kind::f16 instruction descriptor: D = F32, A = B = BF16, both
                            // K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
                            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nn >> 3) << 17) |
                                                   ((uint32_t)(TC_M >> 4) << 24);
                            // start-address field: (offset >> 4) adds without carry (smem < 256 KB)
                            const uint64_t bd = bd0 + (uint64_t)((part * 256 / 8 * 1024 + kk * 256) >> 4);
                            const uint32_t acc = (kk | s) ? 1u : 0u;
                            const uint32_t dt = tmem + (uint32_t)(TC_N * s + 256 * part);
                            if (s < A_TMEM_SLICES) {  // A from TMEM: K = 16 is 8 columns
                                const uint32_t at = tmem + (uint32_t)(A_TCOL + 32 * s + 8 * kk);
                                asm volatile(
                                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                                    " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dt),
                                    "r"(at), "l"(bd), "r"(idesc), "r"(acc)
                                    : "memory");
                            } else {
                                const uint64_t ad =
                                    ad0 + (uint64_t)(((s - A_TMEM_SLICES) * A_SLICE + kk * 256) >> 4);
                                asm volatile(
                                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
                                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                                    : "memory");
                            }
                        }
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(bar_mma + (it & 1)))
                             : "memory");
                ++issued;
                mbar_arrive(bar_ready);
            }
        }
        __syncwarp();
    } else if ((warp & 3) < live_quads) {
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, columns
        // 16 c .. 16 c + 15 with c = (w - 4) / 4; lane u < 16 holds the x row
        // of live shift 16 (w % 4) + u of the group, lane u + 16 its p row.
        // (Warps of a quadrant without live rows skip this loop; the
        // accumulator-free barrier counts only the others.)
        const int q = warp & 3, cg = (warp - EPI_WARP0) >> 2;
        const int r = 32 * q + lane;
        const int which = row_which(r);
        const int pos = g * 64 + row_shift(r);
        const bool live = pos < n_live;
        const int j = live ? a.live[1 + pos] : 0;
        const bool store = live && (which == 0 || a.keep_p);
        const int E = s_rowexp[r];
        const double own = s_rown[r];
        const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(cg * EPI_COLS);
        // this lane's piece of a panel (system j, columns 16 cg .. 16 cg + 15):
        // x rows in X, p rows in Pmat; consecutive panels m * 48 values apart
        double *const pbase =
            live && (which == 0 || a.Pmat) ? (which ? a.Pmat : a.X) + (size_t)j * TC_N + cg * EPI_COLS : nullptr;
        const size_t pstride = (size_t)a.m * TC_N;
        const bool have_p = a.Pmat != nullptr;
        // x and p values of a tile, loaded one tile ahead: the loads are in
        // flight while the warp waits for that tile's MMAs and drains them.
        // 32-byte sector accesses (pieces are 16 values from a 32-byte aligned base)
        double pv[EPI_COLS];
        auto load_pv = [&](unsigned t) {
            const unsigned c0 = t * TC_N + cg * EPI_COLS;
            const double *src = pbase ? pbase + (size_t)t * pstride : nullptr;
            if (src && c0 + EPI_COLS <= n) {
#pragma unroll
                for (int u = 0; u < EPI_COLS; u += 4) ld_sector(src + u, pv[u], pv[u + 1], pv[u + 2], pv[u + 3]);
            } else {
#pragma unroll
                for (int u = 0; u < EPI_COLS; ++u) pv[u] = (src && c0 + u < n) ? src[u] : 0.0;
            }
        };
        if (blockIdx.x < ntiles) load_pv(blockIdx.x);
        int it = 0;
        for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
            // the warp decides as one: tcgen05.ld and the shuffles below are warp-collective
            bool bad = *(volatile int *)s_fail != 0;
            if (!bad)
                bad = !mbar_wait(bar_ready, it & 1, s_fail) || !mbar_wait(bar_mma + (it & 1), (it >> 1) & 1, s_fail);
            if (__any_sync(0xffffffffu, bad)) {
                if (lane == 0) atomicExch(s_fail, 1);
                break;
            }
            tc_fence_after();
            // exact diagonal sums -> floor(T / 2^12)
            long long T[EPI_COLS];
#pragma unroll
            for (int c4 = 0; c4 < EPI_COLS / 4; ++c4) {
                uint32_t dv[NDIAG][4];
#pragma unroll
                for (int d = 0; d < NDIAG; ++d)
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                                 : "=r"(dv[d][0]), "=r"(dv[d][1]), "=r"(dv[d][2]), "=r"(dv[d][3])
                                 : "r"(tbase + (uint32_t)(d * TC_N + 4 * c4)));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    uint32_t B[NDIAG];
#pragma unroll
                    for (int d = 0; d < NDIAG; ++d) B[d] = __float_as_uint(__uint_as_float(dv[d][u]) + MAGIC);
                    T[4 * c4 + u] = diag_sum(B);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar_tfree);

            const unsigned c0 = t * TC_N + cg * EPI_COLS;
            const bool full = c0 + EPI_COLS <= n;
            const int *Fc = s_F + (it & 3) * TC_N + cg * EPI_COLS;
            double *dst = store && pbase ? pbase + (size_t)t * pstride : nullptr;
            // one pass per four columns: round, own-vector terms (x lanes take
            // the old Pmat from their p lane), store
#pragma unroll
            for (int u = 0; u < EPI_COLS; u += 4) {
                double o4[4];
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const double G = E != EXP_NONE ? join_t(T[u + h], E + Fc[u + h] - 56) : 0.0;
                    const double po = __shfl_xor_sync(0xffffffffu, pv[u + h], 16);
                    const double pold = which ? pv[u + h] : (have_p ? po : 0.0);
                    const double y = fma(own, pold, G);
                    o4[h] = which ? y : pv[u + h] + y;
                }
                if (dst) {
                    if (full)
                        st_sector(dst + u, o4[0], o4[1], o4[2], o4[3]);
                    else {
#pragma unroll
                        for (int h = 0; h < 4; ++h)
                            if (c0 + u + h < n) dst[u + h] = o4[h];
                    }
                }
            }
            if (t + gridDim.x < ntiles) load_pv(t + gridDim.x);
        }
    }
    // every path ends here: let copies and MMAs still in flight after a
    // timeout finish (bounded), then free TMEM
    __syncthreads();
    if (tid == 32 * MMA_WARP && *(volatile int *)s_fail) {
        int dummy = 0;
        if (!a_ok) mbar_wait(bar_a, 0, &dummy);
        if (issued > 0) mbar_wait(bar_mma + ((issued - 1) & 1), ((issued - 1) >> 1) & 1, &dummy);
    }
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
    return 256 + 64 * sizeof(unsigned long long) + (size_t)groups * (A_BYTES + TC_M * (sizeof(int) + sizeof(double))) +
           sizeof(int) * ((size_t)(m > 0 ? m : 0) + 1);
}

int hbk_flush_tc_max_slots(void) { return TC_K; }

// x_j (and p_j when keep_p) from the first L basis slots on the tensor cores,
// for the live shifts only: conv_k[j] == 0 or conv_k[j] > k_last (conv_k
// NULL: every shift).  slot_max: bits of each slot's max |value| (NULL:
// computed here; else [L][HBK_SLOT_SPREAD] partial maxima).  V: [L][ld] slots; X, Pmat: panel-major (HBK_PANEL),
// m systems, 32-byte aligned; ws: device workspace of
// hbk_flush_tc_workspace_bytes(m), err: device int.
int hbk_flush_tc_run_live(const double *V, size_t ld, unsigned n, int L, const double *Xc, const double *Pc, int cap,
                          const double *own, int m, double *X, double *Pmat, int keep_p, const int *conv_k,
                          int k_last, const unsigned long long *slot_max_in, void *ws, int *err, cudaStream_t st) {
    // x and p pieces are accessed in 32-byte sectors: 32-byte aligned arrays
    if (L > TC_K || L < 1 || m < 1 || n == 0 || ld < n || ((uintptr_t)X & 31) || ((uintptr_t)Pmat & 31))
        return (int)cudaErrorInvalidValue;
    const int groups = (m + 63) / 64;
    unsigned char *w = (unsigned char *)ws;
    unsigned long long *slot_max = (unsigned long long *)(w + 256);
    unsigned char *aimg = w + 256 + 64 * sizeof(unsigned long long);
    int *rowexp = (int *)(aimg + (size_t)groups * A_BYTES);
    double *rown = (double *)(rowexp + groups * TC_M);
    int *live = (int *)(rown + (size_t)groups * TC_M);
    cudaError_t e = cudaSuccess;
    k_flush_live<<<1, 32, 0, st>>>(conv_k, m, k_last, live);
    if (slot_max_in) {
        static_assert(HBK_SLOT_SPREAD == 32, "one warp folds a slot's partial maxima");
        k_fold_slot_max<<<L, 32, 0, st>>>(slot_max_in, L, slot_max);
    } else {
        if ((e = cudaMemsetAsync(slot_max, 0, 64 * sizeof(unsigned long long), st))) return (int)e;
        dim3 gs(grid_for(n, 16) < 64 ? grid_for(n, 16) : 64, L);
        k_slot_max<<<gs, NT, 0, st>>>(V, ld, n, L, slot_max);
    }
    k_flush_prep<<<dim3(TC_M, groups), TC_K, 0, st>>>(Xc, Pc, cap, own, L, slot_max, live, aimg, rowexp, rown);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    static unsigned attr_set = 0;  // one bit per device
    if (dev < 32 && !(attr_set & (1u << dev))) {
        e = cudaFuncSetAttribute(k_flush_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e) return (int)e;
        attr_set |= 1u << dev;
    }
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned ntiles = (n + TC_N - 1) / TC_N;
    const unsigned gx = ntiles < (unsigned)sms ? ntiles : (unsigned)sms;
    TcArgs args{V, ld, n, L, slot_max, aimg, rowexp, rown, X, Pmat, m, keep_p, live, err};
    k_flush_tc<<<dim3(gx, groups), TC_THREADS, SMEM_BYTES, st>>>(args);
    return (int)cudaGetLastError();
}

// device address of the live-shift count of the last hbk_flush_tc_run_live on ws
const int *hbk_flush_tc_live_count(const void *ws, int m) {
    const int groups = (m + 63) / 64;
    const unsigned char *w = (const unsigned char *)ws + 256 + 64 * sizeof(unsigned long long) + (size_t)groups * A_BYTES;
    return (const int *)(w + (size_t)groups * TC_M * (sizeof(int) + sizeof(double)));
}

// every shift live
int hbk_flush_tc_run(const double *V, size_t ld, unsigned n, int L, const double *Xc, const double *Pc, int cap,
                     const double *own, int m, double *X, double *Pmat, int keep_p, void *ws, int *err,
                     cudaStream_t st) {
    return hbk_flush_tc_run_live(V, ld, n, L, Xc, Pc, cap, own, m, X, Pmat, keep_p, nullptr, 0, nullptr, ws, err, st);
}

}  // extern "C"
