// COO -> CSR on the GPU, stable within rows.
//
// The reference converts on the host: a stable sort of the triplets by row
// (src/matrix.c:206-242; its own merge sort, so entries of a row keep their
// file order), then one pass that cuts the rows.  Here the same ordering is a
// least-significant-digit radix sort of (row, entry index) pairs on the
// device, 8 bits per pass and only as many passes as the row count needs.
// Each pass: per-tile digit counts, one exclusive scan of the counts in
// digit-major order (digit 0 of every tile, then digit 1, ...), and a scatter
// that is stable inside a tile (each warp walks its part of the tile 32
// entries at a time, in order, ranking equal digits with __match_any_sync).
// Row pointers then come from the sorted rows (each entry writes the pointers
// of the rows that start at it), and columns and values are gathered once.
// Rows or columns out of range set an error flag instead of writing.
#include <stdint.h>

#include "hbk_device.cuh"

using namespace hbk;

namespace {

constexpr int SORT_NT = 256;
constexpr int SORT_WARPS = SORT_NT / 32;
constexpr int PER_THREAD = 16;
constexpr int TILE = SORT_NT * PER_THREAD;  // entries per block and pass
constexpr int WARP_SPAN = TILE / SORT_WARPS;  // 512 entries per warp
constexpr int SCAN_NT = 1024;
constexpr int SCAN_PER = 8;
constexpr int SCAN_CHUNK = SCAN_NT * SCAN_PER;
static_assert(SORT_NT == 256, "one thread per digit value");

// ---- exclusive scan of uint32 (three phases; totals below 2^32)
__device__ __forceinline__ unsigned warp_incl(unsigned v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// exclusive scan of one value per thread over a block of SCAN_NT threads
__device__ __forceinline__ unsigned block_excl(unsigned v, unsigned *s_w, unsigned *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned inc = warp_incl(v);
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    if (w == 0) {
        const unsigned x = lane < SCAN_NT / 32 ? s_w[lane] : 0u;
        const unsigned xi = warp_incl(x);
        if (lane < SCAN_NT / 32) s_w[lane] = xi - x;
        if (lane == SCAN_NT / 32 - 1) s_w[32] = xi;
    }
    __syncthreads();
    const unsigned r = s_w[w] + inc - v;
    if (total) *total = s_w[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_reduce(const unsigned *in, size_t len, unsigned *part) {
    __shared__ unsigned s_w[33];
    const size_t base = (size_t)blockIdx.x * SCAN_CHUNK;
    unsigned v = 0;
#pragma unroll
    for (int u = 0; u < SCAN_PER; ++u) {
        const size_t i = base + (size_t)u * SCAN_NT + threadIdx.x;
        if (i < len) v += in[i];
    }
    unsigned tot;
    block_excl(v, s_w, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// one block: exclusive scan of the per-chunk totals, in place
__global__ void __launch_bounds__(SCAN_NT) k_scan_parts(unsigned *part, unsigned np) {
    __shared__ unsigned s_w[33];
    unsigned carry = 0;
    for (unsigned b = 0; b < np; b += SCAN_NT) {
        const unsigned i = b + threadIdx.x;
        const unsigned v = i < np ? part[i] : 0u;
        unsigned tot;
        const unsigned ex = block_excl(v, s_w, &tot);
        if (i < np) part[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_apply(const unsigned *in, size_t len, const unsigned *part,
                                                        unsigned *out) {
    __shared__ unsigned s_w[33];
    const size_t base = (size_t)blockIdx.x * SCAN_CHUNK + (size_t)threadIdx.x * SCAN_PER;
    unsigned v[SCAN_PER], sum = 0;
#pragma unroll
    for (int u = 0; u < SCAN_PER; ++u) {
        const size_t i = base + u;
        v[u] = i < len ? in[i] : 0u;
        sum += v[u];
    }
    unsigned run = part[blockIdx.x] + block_excl(sum, s_w, nullptr);
#pragma unroll
    for (int u = 0; u < SCAN_PER; ++u) {
        const size_t i = base + u;
        if (i < len) out[i] = run;
        run += v[u];
    }
}

// ---- radix sort passes
__global__ void __launch_bounds__(SORT_NT) k_digit_count(const unsigned *__restrict__ key, unsigned nnz, int shift,
                                                         unsigned nblk, unsigned *counts) {
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * TILE;
#pragma unroll 4
    for (int u = 0; u < PER_THREAD; ++u) {
        const size_t i = base + (size_t)u * SORT_NT + threadIdx.x;
        if (i < nnz) atomicAdd(&h[(key[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// stable scatter of one pass; idx_in == nullptr means the identity (first pass)
__global__ void __launch_bounds__(SORT_NT) k_digit_scatter(const unsigned *__restrict__ key_in,
                                                           const unsigned *__restrict__ idx_in, unsigned nnz,
                                                           int shift, unsigned nblk, const unsigned *__restrict__ offs,
                                                           unsigned *__restrict__ key_out,
                                                           unsigned *__restrict__ idx_out) {
    __shared__ unsigned hw[SORT_WARPS][256];  // per-warp digit counts, then running positions
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < SORT_WARPS * 256; i += SORT_NT) (&hw[0][0])[i] = 0;
    __syncthreads();
    const size_t wbase = (size_t)blockIdx.x * TILE + (size_t)w * WARP_SPAN;
    for (int c = 0; c < WARP_SPAN / 32; ++c) {
        const size_t i = wbase + (size_t)c * 32 + lane;
        if (i < nnz) atomicAdd(&hw[w][(key_in[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    // thread d: the tile's start for digit d, then each warp's start
    {
        const int d = threadIdx.x;
        unsigned pos = offs[(size_t)d * nblk + blockIdx.x];
#pragma unroll
        for (int ww = 0; ww < SORT_WARPS; ++ww) {
            const unsigned cnt = hw[ww][d];
            hw[ww][d] = pos;
            pos += cnt;
        }
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int c = 0; c < WARP_SPAN / 32; ++c) {
        const size_t i = wbase + (size_t)c * 32 + lane;
        const bool valid = i < nnz;
        const unsigned k = valid ? key_in[i] : 0u;
        const unsigned dg = valid ? ((k >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        const unsigned rank = __popc(peers & lt);
        if (valid) {
            const unsigned pos = hw[w][dg] + rank;
            key_out[pos] = k;
            idx_out[pos] = idx_in ? idx_in[i] : (unsigned)i;
        }
        __syncwarp();
        // the highest lane of each group advances its digit's position
        if (valid && (peers >> lane) == 1u) hw[w][dg] += __popc(peers);
        __syncwarp();
    }
}

__global__ void k_check(const unsigned *__restrict__ row, const unsigned *__restrict__ col, unsigned nnz, unsigned n,
                        int *err) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < nnz; i += (size_t)gridDim.x * NT)
        if (row[i] >= n || col[i] >= n) atomicExch(err, 1);
}

// ptr[r] = first position with row >= r, from the sorted rows
__global__ void k_row_ptr(const unsigned *__restrict__ key, unsigned nnz, unsigned n, unsigned *ptr) {
    for (size_t p = blockIdx.x * (size_t)NT + threadIdx.x; p <= nnz; p += (size_t)gridDim.x * NT) {
        // (rows >= n, which k_check reports, are clamped: nothing past ptr[n])
        const long long r = p < nnz && key[p] < n ? (long long)key[p] : (long long)n;
        const long long rp = p > 0 ? (key[p - 1] < n ? (long long)key[p - 1] : (long long)n) : -1ll;
        for (long long q = rp + 1; q <= r; ++q) ptr[q] = (unsigned)p;
    }
}

__global__ void k_gather(const unsigned *__restrict__ perm, const unsigned *__restrict__ col,
                         const double *__restrict__ val, unsigned nnz, unsigned *__restrict__ col_out,
                         double *__restrict__ val_out) {
    for (size_t p = blockIdx.x * (size_t)NT + threadIdx.x; p < nnz; p += (size_t)gridDim.x * NT) {
        const unsigned j = perm[p];
        col_out[p] = col[j];
        val_out[p] = val[j];
    }
}

int scan_excl(const unsigned *in, size_t len, unsigned *out, unsigned *part, cudaStream_t st) {
    if (!len) return 0;
    const unsigned nb = (unsigned)((len + SCAN_CHUNK - 1) / SCAN_CHUNK);
    k_scan_reduce<<<nb, SCAN_NT, 0, st>>>(in, len, part);
    k_scan_parts<<<1, SCAN_NT, 0, st>>>(part, nb);
    k_scan_apply<<<nb, SCAN_NT, 0, st>>>(in, len, part, out);
    return (int)cudaGetLastError();
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

size_t hbk_coo_to_csr_tmp_bytes(unsigned nnz) {
    const size_t nblk = (nnz + TILE - 1) / TILE + 1;
    const size_t cnt = 256 * nblk;
    const size_t parts = (cnt + SCAN_CHUNK - 1) / SCAN_CHUNK + 1;
    return 4 * align256(sizeof(unsigned) * ((size_t)nnz + 1)) + 2 * align256(sizeof(unsigned) * cnt) +
           align256(sizeof(unsigned) * parts) + 256;
}

// ptr [n+1], col_out/val_out [nnz] from device COO triplets; tmp of
// hbk_coo_to_csr_tmp_bytes(nnz) bytes; err: device int set to 1 when a row
// or column index is >= n (the output is then not meaningful).
int hbk_coo_to_csr(unsigned n, unsigned nnz, const unsigned *row, const unsigned *col, const double *val,
                   unsigned *ptr, unsigned *col_out, double *val_out, void *tmp, int *err, cudaStream_t st) {
    const unsigned nblk = (nnz + TILE - 1) / TILE;
    const size_t cnt = (size_t)256 * (nblk ? nblk : 1);
    unsigned char *t = (unsigned char *)tmp;
    unsigned *keyA = (unsigned *)t;
    t += align256(sizeof(unsigned) * ((size_t)nnz + 1));
    unsigned *keyB = (unsigned *)t;
    t += align256(sizeof(unsigned) * ((size_t)nnz + 1));
    unsigned *idxA = (unsigned *)t;
    t += align256(sizeof(unsigned) * ((size_t)nnz + 1));
    unsigned *idxB = (unsigned *)t;
    t += align256(sizeof(unsigned) * ((size_t)nnz + 1));
    unsigned *counts = (unsigned *)t;
    t += align256(sizeof(unsigned) * cnt);
    unsigned *offs = (unsigned *)t;
    t += align256(sizeof(unsigned) * cnt);
    unsigned *part = (unsigned *)t;

    const int g = grid_for(nnz ? nnz : 1, 4);
    k_check<<<g, NT, 0, st>>>(row, col, nnz, n, err);
    int passes = 0;
    for (unsigned long long top = n ? n - 1 : 0; top; top >>= 8) ++passes;
    if (passes == 0) passes = 1;
    const unsigned *kin = row, *iin = nullptr;
    unsigned *kout = keyA, *iout = idxA;
    for (int ps = 0; ps < passes && nnz; ++ps) {
        k_digit_count<<<nblk, SORT_NT, 0, st>>>(kin, nnz, 8 * ps, nblk, counts);
        int e = scan_excl(counts, (size_t)256 * nblk, offs, part, st);
        if (e) return e;
        k_digit_scatter<<<nblk, SORT_NT, 0, st>>>(kin, iin, nnz, 8 * ps, nblk, offs, kout, iout);
        kin = kout;
        iin = iout;
        kout = (kout == keyA) ? keyB : keyA;
        iout = (iout == idxA) ? idxB : idxA;
    }
    const unsigned *skey = nnz ? kin : row;
    k_row_ptr<<<grid_for(nnz + 1, 4), NT, 0, st>>>(skey, nnz, n, ptr);
    if (nnz) k_gather<<<g, NT, 0, st>>>(iin, col, val, nnz, col_out, val_out);
    return (int)cudaGetLastError();
}

}  // extern "C"
