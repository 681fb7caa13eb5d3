// Device helpers shared by the solver's kernels: deterministic block
// reductions, the last-block ticket, and the row-block CSR SpMV core.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hbk.h"

namespace hbk {

constexpr int NT = HBK_THREADS;

// Blocks per SM that the kernels taking the HYB form are compiled for (the
// other forms keep the compiler's choice).  The HYB products are
// latency-bound, and all HYB kernels share one warp-list plan sized for the
// smallest one-wave grid among them.  Measured on GB300, config 3 (2 M
// power-law rows): with K1 and K3 at 8 blocks (32 registers, a few bytes
// spilled) the solve took as long as with them at 4 blocks (56 registers),
// and the plain product, at the full wave of 8 blocks, took 0.166 against
// 0.184 ms.
#ifndef HBK_HYB_MINB
#define HBK_HYB_MINB 8
#endif
constexpr int NW = NT / 32;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block with a fixed tree (same order on every run); every
// thread gets the total.  `sh` needs NW doubles.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = (l < NW) ? sh[l] : 0.0;
    return warp_sum(t);
}

__device__ __forceinline__ double2 block_sum2(double2 v, double *sh) {
    v.x = warp_sum(v.x);
    v.y = warp_sum(v.y);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) {
        sh[w] = v.x;
        sh[NW + w] = v.y;
    }
    __syncthreads();
    double2 t;
    t.x = warp_sum((l < NW) ? sh[l] : 0.0);
    t.y = warp_sum((l < NW) ? sh[NW + l] : 0.0);
    return t;
}

// Writes this block's partial(s) and takes a ticket; returns true in every
// thread of the block that arrives last of `nb` blocks (the launch's grid by
// default).  That block then sums the partials in block-index order (fixed
// tree), so results do not depend on timing.
__device__ __forceinline__ bool take_ticket(unsigned *counter, unsigned nb) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == nb - 1);
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}
__device__ __forceinline__ bool take_ticket(unsigned *counter) { return take_ticket(counter, gridDim.x); }

// Which block of how many: the launch's own grid (HwGrid), or a virtual grid
// of `vnb` blocks that one CTA of a persistent launch plays in turn (VGrid).
// Loads of vectors that the same launch also writes go through ld/ldx: a
// plain load (and the read-only path for the SpMV gather) in a kernel that
// runs one step, an L2 load in a persistent kernel, where the read-only
// cache may still hold a value from an earlier step.
struct HwGrid {
    static constexpr bool hw = true;
    __device__ __forceinline__ unsigned b() const { return blockIdx.x; }
    __device__ __forceinline__ unsigned nb() const { return gridDim.x; }
    template <class T>
    __device__ static __forceinline__ T ld(const T *p) { return *p; }
    template <class T>
    __device__ static __forceinline__ T ldx(const T *p) { return __ldg(p); }
    template <class T>
    __device__ static __forceinline__ T ldv(const T *p) { return __ldg(p); }
};
// element i of a vector the launch also writes (p indexed directly in a
// one-step kernel, so its code is what it was without grid views)
#define HBK_LD(G, p, i) ((G::hw) ? (p)[i] : __ldcg((p) + (i)))

template <class G>
struct is_hw_grid {
    static constexpr bool value = false;
};
template <>
struct is_hw_grid<HwGrid> {
    static constexpr bool value = true;
};
struct VGrid {
    static constexpr bool hw = false;
    unsigned vb, vnb;
    __device__ __forceinline__ unsigned b() const { return vb; }
    __device__ __forceinline__ unsigned nb() const { return vnb; }
    template <class T>
    __device__ static __forceinline__ T ld(const T *p) { return __ldcg(p); }
    template <class T>
    __device__ static __forceinline__ T ldx(const T *p) { return __ldcg(p); }
    // matrix values: the seed's private SELL-32 copy gets a new diagonal after
    // a seed switch, inside the same persistent launch
    template <class T>
    __device__ static __forceinline__ T ldv(const T *p) { return __ldcg(p); }
};

// Called by the last block: sums partials[0..nparts) in a fixed order.
__device__ __forceinline__ double sum_partials(const double *partials, int nparts, double *sh) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += NT) acc += __ldcg(partials + i);
    return block_sum(acc, sh);
}

__device__ __forceinline__ bool fin(double v) { return isfinite(v) != 0; }

// max of v over the block (every thread calls), then one atomicMax into
// out[blockIdx.x % HBK_SLOT_SPREAD] when it is nonzero (bits of non-negative
// doubles order as unsigned integers; spreading the blocks over entries keeps
// the atomics from queueing on one address); `sh` needs NW values
__device__ __forceinline__ void block_max_to(unsigned long long v, unsigned long long *sh, unsigned long long *out) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = 0;
        for (int i = 0; i < NW; ++i) m = sh[i] > m ? sh[i] : m;
        if (m) atomicMax(out + blockIdx.x % HBK_SLOT_SPREAD, m);
    }
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// index of element i of system j in a panel-major array of m systems
__device__ __forceinline__ size_t panel_idx(int j, unsigned i, int m) {
    const unsigned p = i / HBK_PANEL;
    return ((size_t)p * (unsigned)m + (unsigned)j) * HBK_PANEL + (i - p * HBK_PANEL);
}

// ---------------------------------------------------------------------------
// Row-block CSR SpMV core.
//
// Rows are cut on the host into blocks (hbk_plan_rows): a TILE block holds up
// to NT consecutive short rows with at most HBK_TILE_NNZ nonzeros in total; a
// LONG block holds one row.  A persistent grid walks the blocks in order.  For
// a TILE block the CTA stages the block's values and the gathered x values in
// shared memory with coalesced loads, then each thread sums one row in stored
// order with FMAs (the same order as the reference's row loop,
// src/openmp_matrix.c:47-58).  A LONG row is summed by the whole CTA with a
// fixed tree.  `epi(row, acc)` finishes each row; it runs once per row.
// ---------------------------------------------------------------------------
struct SpmvSmem {
    double val[HBK_TILE_NNZ];
    double xv[HBK_TILE_NNZ];
    double red[2 * NW];
};

// SELL-32 path: one thread per row, the 32 rows of a slice in one warp.  Entry
// e of the slice's rows is one 256-byte line of values and one 128-byte line
// of column indices, so every load is coalesced and no shared memory or
// barrier is needed; each row is still summed in stored order with FMAs from
// 0, exactly as in the TILE path (padding entries are skipped by row length).
template <class Epi, class G = HwGrid>
__device__ __forceinline__ void spmv_rows_sell(const hbk_matrix &A, const double *__restrict__ x, Epi &epi,
                                               const G &g = G()) {
    const unsigned *__restrict__ ptr = A.ptr;
    const double *__restrict__ sval = A.sval;
    const unsigned *__restrict__ scol = A.scol;
    const unsigned n = A.n;
    const unsigned ns = (n + 31) / 32;
    const unsigned stride = g.nb() * NT;
    for (unsigned r0 = g.b() * NT; r0 < n; r0 += stride) {
        const unsigned r = r0 + threadIdx.x;
        const unsigned s = r >> 5, lane = r & 31;
        unsigned long long base = 0;
        unsigned w = 0;
        if (s < ns) {
            base = __ldg(A.sptr + s);
            w = (unsigned)((__ldg(A.sptr + s + 1) - base) >> 5);
        }
        const unsigned len = r < n ? __ldg(ptr + r + 1) - __ldg(ptr + r) : 0;
        const double *__restrict__ vv = sval + base + lane;
        const unsigned *__restrict__ cc = scol + base + lane;
        double acc = 0.0;
#pragma unroll 4
        for (unsigned e = 0; e < w; ++e) {
            if (e < len) acc = fma(G::ldv(vv + 32 * (size_t)e), G::ldx(x + __ldg(cc + 32 * (size_t)e)), acc);
        }
        if (r < n) epi(r, acc);
    }
}

template <class Epi>
__device__ __forceinline__ void spmv_rows_tile(const hbk_matrix &A, const double *__restrict__ x, Epi &epi,
                                               SpmvSmem &sm) {
    const unsigned *__restrict__ ptr = A.ptr;
    const unsigned *__restrict__ col = A.col;
    const double *__restrict__ val = A.val;
    for (unsigned b = blockIdx.x; b < A.nblk; b += gridDim.x) {
        const unsigned r0 = __ldg(A.blk_row + b), r1 = __ldg(A.blk_row + b + 1);
        const unsigned e0 = __ldg(ptr + r0), e1 = __ldg(ptr + r1);
        if (__ldg(A.blk_kind + b) == HBK_BLK_LONG) {
            double acc = 0.0;
            for (unsigned e = e0 + threadIdx.x; e < e1; e += NT) acc = fma(__ldg(val + e), __ldg(x + __ldg(col + e)), acc);
            acc = block_sum(acc, sm.red);
            if (threadIdx.x == 0) epi(r0, acc);
            __syncthreads();
            continue;
        }
        const unsigned cnt = e1 - e0;
        for (unsigned e = threadIdx.x; e < cnt; e += NT) {
            const unsigned c = __ldg(col + e0 + e);
            sm.val[e] = __ldg(val + e0 + e);
            sm.xv[e] = __ldg(x + c);
        }
        __syncthreads();
        const unsigned r = r0 + threadIdx.x;
        if (r < r1) {
            const unsigned a = __ldg(ptr + r) - e0, z = __ldg(ptr + r + 1) - e0;
            double acc = 0.0;
            for (unsigned e = a; e < z; ++e) acc = fma(sm.val[e], sm.xv[e], acc);
            epi(r, acc);
        }
        __syncthreads();
    }
}

// HYB path: persistent warps over work items.  Long rows (more than
// HBK_HYB_SHORT entries, longest first) take g lanes each: 32 (one row per
// item) above HBK_HYB_L16 entries, 16 (two rows of similar length per item)
// above HBK_HYB_L4, else 4 (eight rows per item).  Lane j of a row's group
// sums entries j, j + g, ... in stored order with FMAs, and the g partial
// sums meet in a fixed shuffle tree (log2 g FP64 adds, instead of 5 for every
// row).  Short rows are in SELL-32 slices, one warp each, whose 32 rows were
// sorted by length inside a window of HBK_HYB_WINDOW rows, so the lanes of a
// warp have similar row lengths (an FP64 instruction costs the same whatever
// its active lanes); each short row is summed in stored order with FMAs from
// 0, as in the other paths.  The host deals the items to A.hnw warp lists,
// costliest first, each to the list with the least work so far (cost: a
// header, one step per g entries of the group's longest row or per entry of
// a slice, and the tree), so no warp is left with several of the longest
// rows; warp w of the grid runs lists w, w + (warps of the grid), ...  A row's
// arithmetic does not depend on the list it is in.
template <class Epi>
__device__ __forceinline__ void spmv_rows_hyb(const hbk_matrix &A, const double *__restrict__ x, Epi &epi) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned nw = (gridDim.x * NT) >> 5;
    for (unsigned w = (blockIdx.x * NT + threadIdx.x) >> 5; w < A.hnw; w += nw) {
        const unsigned k1 = __ldg(A.hwbeg + w + 1);
        for (unsigned k = __ldg(A.hwbeg + w); k < k1; ++k) {
            const unsigned it = __ldg(A.hitem + k);
            if (it < A.hitl) {
                unsigned g, i, iend;
                if (it < A.hit16) {
                    g = 32;
                    i = it;
                    iend = A.hrow32;
                } else if (it < A.hit4) {
                    g = 16;
                    i = A.hrow32 + 2 * (it - A.hit16) + (lane >> 4);
                    iend = A.hrow16;
                } else {
                    g = 4;
                    i = A.hrow16 + 8 * (it - A.hit4) + (lane >> 2);
                    iend = A.nwrow;
                }
                const bool valid = i < iend;
                uint2 rg = make_uint2(0u, 0u);
                unsigned r = 0;
                if (valid) {
                    rg = __ldg(reinterpret_cast<const uint2 *>(A.wrng) + i);
                    r = __ldg(A.wrow + i);
                }
                double acc = 0.0;
                for (unsigned e = rg.x + (lane & (g - 1)); e < rg.y; e += g)
                    acc = fma(__ldg(A.val + e), __ldg(x + __ldg(A.col + e)), acc);
                for (unsigned o = g >> 1; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (valid && (lane & (g - 1)) == 0) epi(r, acc);
            } else {
                const unsigned s = it - A.hitl;
                const unsigned long long base = __ldg(A.sptr + s);
                const unsigned wd = (unsigned)((__ldg(A.sptr + s + 1) - base) >> 5);
                const unsigned r = __ldg(A.srow + 32 * (size_t)s + lane);
                const unsigned len = __ldg(A.slen + 32 * (size_t)s + lane);
                const double *__restrict__ vv = A.sval + base + lane;
                const unsigned *__restrict__ cc = A.scol + base + lane;
                double acc = 0.0;
#pragma unroll 4
                for (unsigned e = 0; e < wd; ++e)
                    if (e < len) acc = fma(__ldg(vv + 32 * (size_t)e), __ldg(x + __ldg(cc + 32 * (size_t)e)), acc);
                if (r < A.n) epi(r, acc);
            }
        }
    }
}

// MERGE path: nonzero-balanced work (merge-path decomposition), one warp per
// work unit.  The host cuts the rows of at most HBK_MERGE_LONG entries into
// blocks of consecutive rows with rows + nonzeros <= HBK_MERGE_ITEMS (32
// lanes x HBK_MERGE_IPT items) and lists the longer rows apart (longest
// first).  Units, in order: the long rows (one warp each: four FMA chains per
// lane, entries in stored order within a chain, then a fixed tree), then the
// blocks; unit u goes to warp u mod (warps of the grid), so no warp waits for
// another and the assignment, hence every sum, is the same on every run.  A
// block is staged in the warp's own shared memory with coalesced loads
// (values, the gathered x values, the row end offsets; a lane's loads all
// issue before the first is used); lane l then walks items [l IPT, (l + 1)
// IPT) of the merge of the row ends with the nonzeros, so every lane gets the
// same number of (row end + nonzero) items whatever the row lengths.  A row
// that starts and ends inside one lane is summed by that lane in stored order
// with FMAs from 0 (the other paths' arithmetic); a row cut between lanes is
// the sum of its pieces (each an FMA chain in stored order) over a fixed
// shuffle tree.  The row values are then written to shared memory and
// `epi(row, acc)` runs once per row, in row order across the lanes.
// Item e of a block (and row q's value) sits at e + e / 8: one pad slot per 8
// items, so that the walk, where lane l reads items 8 l .. 8 l + 7, reads
// 72 bytes apart across lanes (no shared-memory bank conflicts) instead of 64.
__device__ __forceinline__ unsigned merge_pad(unsigned e) { return e + (e >> 3); }
constexpr int MERGE_PADDED = HBK_MERGE_ITEMS + HBK_MERGE_ITEMS / 8;
struct MergeWarpSmem {
    double val[MERGE_PADDED];
    double xv[MERGE_PADDED];         // gathered x; after the walk, the rows' values
    unsigned rend[HBK_MERGE_ITEMS];  // end of each row of the block, relative to its first nonzero
};
struct MergeSmem {
    MergeWarpSmem w[NW];
};

constexpr unsigned kNoRow = 0x80000000u;

template <class Epi>
__device__ __forceinline__ void spmv_rows_merge(const hbk_matrix &A, const double *__restrict__ x, Epi &epi,
                                                MergeSmem &sm) {
    constexpr int IPT = HBK_MERGE_IPT;
    const unsigned *__restrict__ ptr = A.ptr;
    const unsigned *__restrict__ col = A.col;
    const double *__restrict__ val = A.val;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    MergeWarpSmem &ws = sm.w[warp];
    const unsigned nwarps = gridDim.x * NW;
    const unsigned units = A.nmlong + A.nmblk;
    for (unsigned u = blockIdx.x * NW + warp; u < units; u += nwarps) {
        if (u < A.nmlong) {
            const unsigned r = __ldg(A.mlong + u);
            const unsigned e0 = __ldg(ptr + r), e1 = __ldg(ptr + r + 1);
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            for (unsigned e = e0 + lane; e < e1; e += 128) {
                const bool h1 = e + 32 < e1, h2 = e + 64 < e1, h3 = e + 96 < e1;
                const unsigned c0 = __ldg(col + e), c1 = h1 ? __ldg(col + e + 32) : 0u;
                const unsigned c2 = h2 ? __ldg(col + e + 64) : 0u, c3 = h3 ? __ldg(col + e + 96) : 0u;
                const double v0 = __ldg(val + e), v1 = h1 ? __ldg(val + e + 32) : 0.0;
                const double v2 = h2 ? __ldg(val + e + 64) : 0.0, v3 = h3 ? __ldg(val + e + 96) : 0.0;
                const double x0 = __ldg(x + c0), x1 = h1 ? __ldg(x + c1) : 0.0;
                const double x2 = h2 ? __ldg(x + c2) : 0.0, x3 = h3 ? __ldg(x + c3) : 0.0;
                a0 = fma(v0, x0, a0);
                if (h1) a1 = fma(v1, x1, a1);
                if (h2) a2 = fma(v2, x2, a2);
                if (h3) a3 = fma(v3, x3, a3);
            }
            const double acc = warp_sum((a0 + a1) + (a2 + a3));
            if (lane == 0) epi(r, acc);
            continue;
        }
        const unsigned b = u - A.nmlong;
        const unsigned r0 = __ldg(A.mblk + 2 * b), r1 = __ldg(A.mblk + 2 * b + 1);
        const unsigned e0 = __ldg(ptr + r0);
        const unsigned nr = r1 - r0, nz = __ldg(ptr + r1) - e0;
        {
            unsigned c[IPT], re[IPT];
            double v[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const unsigned e = lane + 32u * k;
                c[k] = e < nz ? __ldg(col + e0 + e) : 0u;
                v[k] = e < nz ? __ldg(val + e0 + e) : 0.0;
                re[k] = e < nr ? __ldg(ptr + r0 + e + 1) : 0u;
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const unsigned e = lane + 32u * k;
                if (e < nz) {
                    ws.xv[merge_pad(e)] = __ldg(x + c[k]);
                    ws.val[merge_pad(e)] = v[k];
                }
                if (e < nr) ws.rend[e] = re[k] - e0;
            }
        }
        __syncwarp();
        const unsigned tot = nr + nz;
        const unsigned d0 = min(lane * (unsigned)IPT, tot);
        const unsigned d1 = min(d0 + (unsigned)IPT, tot);
        // merge-path search: i row ends and d0 - i nonzeros precede item d0
        unsigned lo = d0 > nz ? d0 - nz : 0, hi = min(d0, nr);
        while (lo < hi) {
            const unsigned mid = (lo + hi) >> 1;
            if (ws.rend[mid] <= d0 - 1 - mid) lo = mid + 1;
            else hi = mid;
        }
        unsigned i = lo, e = d0 - lo;
        // the lane starts inside row i when entries of that row precede e
        bool head = e > (i ? ws.rend[i - 1] : 0u), open = false;
        unsigned head_row = kNoRow;
        double head_v = 0.0, acc = 0.0;
        unsigned rr[IPT];
        double rv[IPT];
#pragma unroll
        for (int q = 0; q < IPT; ++q) {
            rr[q] = kNoRow;
            rv[q] = 0.0;
            const bool valid = d0 + q < d1;
            const bool is_end = valid && i < nr && ws.rend[i] <= e;
            if (is_end) {
                if (head) {
                    head_row = i;
                    head_v = acc;
                    head = false;
                } else {
                    rr[q] = i;
                    rv[q] = acc;
                }
                acc = 0.0;
                open = false;
                ++i;
            } else if (valid) {
                acc = fma(ws.val[merge_pad(e)], ws.xv[merge_pad(e)], acc);
                ++e;
                open = true;
            }
        }
        // pieces of rows cut between lanes: segmented inclusive scan of the
        // open (tail) pieces keyed by row, with as many steps as the longest
        // chain of lanes needs
        const unsigned key = open ? i : (kNoRow | lane);
        double s = open ? acc : 0.0;
        const unsigned kprev = __shfl_up_sync(0xffffffffu, key, 1);
        bool f = lane == 0 || kprev != key;  // a run of the key starts here
#pragma unroll 1
        for (int dd = 1; dd < 32; dd <<= 1) {
            if (__all_sync(0xffffffffu, f)) break;
            const double so = __shfl_up_sync(0xffffffffu, s, dd);
            const bool fo = __shfl_up_sync(0xffffffffu, f, dd);
            if ((int)lane >= dd && !f) {
                s = so + s;
                f = fo;
            }
        }
        const unsigned pk = __shfl_up_sync(0xffffffffu, key, 1);
        const double ps = __shfl_up_sync(0xffffffffu, s, 1);
        __syncwarp();  // every lane is done with the staged values
#pragma unroll
        for (int q = 0; q < IPT; ++q)
            if (rr[q] != kNoRow) ws.xv[merge_pad(rr[q])] = rv[q];
        if (head_row != kNoRow) ws.xv[merge_pad(head_row)] = ((lane > 0 && pk == head_row) ? ps : 0.0) + head_v;
        __syncwarp();
        for (unsigned q = lane; q < nr; q += 32) epi(r0 + q, ws.xv[merge_pad(q)]);
        __syncwarp();  // before the next unit overwrites this warp's staging
    }
}

// Format chosen at compile time so the SELL kernels carry no shared-memory
// tile (full occupancy); launchers pick the instantiation from A.fmt.
// (the virtual grids of a persistent launch take the SELL-32 form only)
template <int FMT, class Epi, class G = HwGrid>
__device__ __forceinline__ void spmv_rows(const hbk_matrix &A, const double *__restrict__ x, Epi &epi,
                                          const G &g = G()) {
    static_assert(FMT == HBK_FMT_SELL || is_hw_grid<G>::value, "virtual grids take the SELL-32 form only");
    if constexpr (FMT == HBK_FMT_SELL) {
        spmv_rows_sell(A, x, epi, g);
    } else if constexpr (FMT == HBK_FMT_HYB) {
        spmv_rows_hyb(A, x, epi);
    } else if constexpr (FMT == HBK_FMT_MERGE) {
        __shared__ MergeSmem sm;
        spmv_rows_merge(A, x, epi, sm);
    } else {
        __shared__ SpmvSmem sm;
        spmv_rows_tile(A, x, epi, sm);
    }
}

// launch helper: kernel<FMT> for the matrix's format
#define HBK_LAUNCH_FMT(A, kern, grid, block, stream, ...)                                   \
    do {                                                                                    \
        if ((A).fmt == HBK_FMT_SELL) kern<HBK_FMT_SELL><<<grid, block, 0, stream>>>(__VA_ARGS__); \
        else if ((A).fmt == HBK_FMT_HYB) kern<HBK_FMT_HYB><<<grid, block, 0, stream>>>(__VA_ARGS__); \
        else if ((A).fmt == HBK_FMT_MERGE) kern<HBK_FMT_MERGE><<<grid, block, 0, stream>>>(__VA_ARGS__); \
        else kern<HBK_FMT_TILE><<<grid, block, 0, stream>>>(__VA_ARGS__);                  \
    } while (0)

// number of SMs of the current device (cached: one device type per process)
inline int sm_count() {
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return sms;
}

// At most one wave of a grid-stride kernel K: the blocks of NT threads that
// are resident on all SMs at once (more blocks only add a partial second wave).
template <auto K>
inline int wave_grid(int want) {
    static const int one_wave = [] {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K, NT, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
        return per_sm * sm_count();
    }();
    return want < one_wave ? want : one_wave;
}

inline int grid_for(unsigned n, int per_thread) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    long need = ((long)n + (long)NT * per_thread - 1) / ((long)NT * per_thread);
    long cap = (long)sms * 8;
    if (cap > HBK_MAX_GRID) cap = HBK_MAX_GRID;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

}  // namespace hbk
