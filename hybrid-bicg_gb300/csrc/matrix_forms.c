/* Matrices of the GB300 solver: upload, the three SpMV forms (CSR row-block
 * tiles, SELL-32, HYB) built on the device from the CSR arrays, the
 * host-pointer product behind matrix.h, and the SpMV-form autotuner with its
 * cache file. */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fcntl.h>
#include <pthread.h>
#include <sys/stat.h>
#include <unistd.h>

#include "host_internal.h"
#include "solver.h"

static int cmp_u64(const void *a, const void *b) {
    const unsigned long long x = *(const unsigned long long *)a, y = *(const unsigned long long *)b;
    return x < y ? -1 : x > y;
}

/* HYB work lists: work items (use_hyb lists them) with their costs, dealt in order of
 * decreasing cost (ties: lower item first), each to the list with the least
 * cost so far (ties: lower list); every list keeps the order of dealing.
 * hwbeg[hnw + 1], hitem[ni]. */
typedef struct {
    unsigned long long load;
    unsigned w;
} hyb_slot;

static int slot_less(const hyb_slot *a, const hyb_slot *b) {
    return a->load < b->load || (a->load == b->load && a->w < b->w);
}

int hbicg__hyb_plan(size_t ni, const unsigned *cost, unsigned hnw, unsigned *hwbeg, unsigned *hitem) {
    unsigned long long *key = malloc(sizeof *key * (ni + 1));
    hyb_slot *h = malloc(sizeof *h * hnw);
    unsigned *owner = malloc(sizeof *owner * (ni + 1));
    unsigned *pos = malloc(sizeof *pos * hnw);
    if (!key || !h || !owner || !pos) {
        free(key);
        free(h);
        free(owner);
        free(pos);
        return HBICG_E_NOMEM;
    }
    for (size_t i = 0; i < ni; ++i) key[i] = ((0xFFFFFFFFull - cost[i]) << 32) | i; /* costliest first, then by item */
    qsort(key, ni, sizeof *key, cmp_u64);
    for (unsigned w = 0; w < hnw; ++w) h[w] = (hyb_slot){0, w}; /* all zero: a valid heap */
    memset(hwbeg, 0, sizeof *hwbeg * ((size_t)hnw + 1));
    for (size_t k = 0; k < ni; ++k) {
        const unsigned i = (unsigned)(key[k] & 0xFFFFFFFFu);
        owner[i] = h[0].w;
        hwbeg[h[0].w + 1]++;
        h[0].load += 0xFFFFFFFFull - (key[k] >> 32);
        for (size_t p = 0;;) { /* sift the grown root down */
            const size_t l = 2 * p + 1, r = l + 1;
            size_t m = p;
            if (l < hnw && slot_less(&h[l], &h[m])) m = l;
            if (r < hnw && slot_less(&h[r], &h[m])) m = r;
            if (m == p) break;
            const hyb_slot t = h[p];
            h[p] = h[m];
            h[m] = t;
            p = m;
        }
    }
    for (unsigned w = 0; w < hnw; ++w) hwbeg[w + 1] += hwbeg[w];
    /* fill each list in the order of dealing */
    memcpy(pos, hwbeg, sizeof *pos * hnw);
    for (size_t k = 0; k < ni; ++k) {
        const unsigned i = (unsigned)(key[k] & 0xFFFFFFFFu);
        hitem[pos[owner[i]]++] = i;
    }
    free(key);
    free(h);
    free(owner);
    free(pos);
    return HBICG_OK;
}

/* HYB: rows of at most HBK_HYB_SHORT entries in SELL-32 slices, sorted by
 * length (longest first, stable) inside windows of HBK_HYB_WINDOW consecutive
 * rows, so that the 32 rows of a slice have similar lengths and the rows a
 * warp writes stay inside one window; each window's list is padded to whole
 * slices with empty lanes.  Longer rows go to a list, longest first, one warp
 * each.  For power-law row lengths (most rows short, a few thousands long),
 * where a thread per row leaves most lanes of a warp idle.  The lengths of the
 * slice rows are kept as bytes after the lane -> row map, so that a warp reads
 * its 32 lengths in one line instead of 64 scattered row pointers.  One
 * allocation holds each long row's entry range, the long rows, and the warp
 * work lists (hbicg__hyb_plan) for one wave of the kernels that take this form. */
static int build_hyb(hbicg_matrix *A, const unsigned *h_ptr, unsigned n) {
    cudaStream_t st = A->ctx->stream;
    if (!n || A->d_hval) return HBICG_OK;
    size_t cap = 0, nw = 0;
    for (unsigned w0 = 0; w0 < n; w0 += HBK_HYB_WINDOW) {
        const unsigned w1 = n - w0 < HBK_HYB_WINDOW ? n : w0 + HBK_HYB_WINDOW;
        unsigned cnt = 0;
        for (unsigned r = w0; r < w1; ++r) {
            if (h_ptr[r + 1] - h_ptr[r] <= HBK_HYB_SHORT)
                cnt++;
            else
                nw++;
        }
        cap += (cnt + 31) / 32 * 32;
    }
    const size_t ns = cap / 32;
    /* lane -> row map (cap + 1 entries), then the lanes' row lengths as bytes */
    const size_t srow_bytes = sizeof(unsigned) * (cap + 1) + cap + 1;
    unsigned *srow = malloc(srow_bytes);
    unsigned long long *wkey = malloc(sizeof(unsigned long long) * (nw + 1));
    /* grid of the HYB kernels: one wave of the heaviest, so every warp of a
     * launch runs exactly one list */
    int hgrid = hbk_spmv_grid((n + HBK_THREADS - 1) / HBK_THREADS);
    {
        const int wf = hbk_hyb_wave_fused(), wb = hbk_hyb_wave_blas();
        if (wf < hgrid) hgrid = wf;
        if (wb < hgrid) hgrid = wb;
        if (hgrid < 1) hgrid = 1;
    }
    const unsigned hnw = (unsigned)hgrid * (HBK_THREADS / 32);
    /* long rows by lanes per row (longest first, so each class is a range) */
    size_t r32 = 0, r16 = 0;
    for (unsigned r = 0; r < n; ++r) {
        const unsigned len = h_ptr[r + 1] - h_ptr[r];
        r32 += len > HBK_HYB_L16;
        r16 += len > HBK_HYB_L4;
    }
    const size_t it16 = r32, it4 = it16 + (r16 - r32 + 1) / 2, itl = it4 + (nw - r16 + 7) / 8;
    const size_t ni = itl + ns;
    /* [2 nw] entry ranges, [nw] rows, [hnw + 1] list starts, [ni] items */
    const size_t plan_words = 3 * nw + hnw + 1 + ni;
    unsigned *wrng = malloc(sizeof(unsigned) * plan_words);
    unsigned *wrow = wrng ? wrng + 2 * nw : NULL;
    unsigned *cost = malloc(sizeof(unsigned) * (ni + 1));
    unsigned long long *sp = malloc(sizeof(unsigned long long) * (ns + 1));
    int rc = HBICG_OK;
    if (!srow || !wkey || !wrng || !cost || !sp) {
        rc = HBICG_E_NOMEM;
        goto done;
    }
    {
        size_t o = 0, wi = 0;
        for (unsigned w0 = 0; w0 < n; w0 += HBK_HYB_WINDOW) {
            const unsigned w1 = n - w0 < HBK_HYB_WINDOW ? n : w0 + HBK_HYB_WINDOW;
            unsigned cnt[HBK_HYB_SHORT + 1] = {0}, pos[HBK_HYB_SHORT + 1];
            for (unsigned r = w0; r < w1; ++r) {
                const unsigned len = h_ptr[r + 1] - h_ptr[r];
                if (len <= HBK_HYB_SHORT)
                    cnt[len]++;
                else /* longest first, then by row: sort the complement of the length */
                    wkey[wi++] = ((unsigned long long)(0xFFFFFFFFu - len) << 32) | r;
            }
            unsigned acc = 0;
            for (int L = HBK_HYB_SHORT; L >= 0; --L) {
                pos[L] = acc;
                acc += cnt[L];
            }
            for (unsigned r = w0; r < w1; ++r) {
                const unsigned len = h_ptr[r + 1] - h_ptr[r];
                if (len <= HBK_HYB_SHORT) srow[o + pos[len]++] = r;
            }
            o += acc;
            while (o % 32) srow[o++] = 0xFFFFFFFFu; /* empty lane */
        }
        unsigned char *slen = (unsigned char *)(srow + cap + 1);
        for (size_t i = 0; i < cap; ++i)
            slen[i] = srow[i] < n ? (unsigned char)(h_ptr[srow[i] + 1] - h_ptr[srow[i]]) : 0;
        qsort(wkey, nw, sizeof *wkey, cmp_u64);
        for (size_t i = 0; i < nw; ++i) {
            const unsigned r = (unsigned)(wkey[i] & 0xFFFFFFFFu);
            wrow[i] = r;
            wrng[2 * i] = h_ptr[r];
            wrng[2 * i + 1] = h_ptr[r + 1];
        }
        sp[0] = 0;
        for (size_t s = 0; s < ns; ++s) {
            unsigned w = 0;
            for (int l = 0; l < 32; ++l) {
                const unsigned r = srow[32 * s + l];
                if (r < n && h_ptr[r + 1] - h_ptr[r] > w) w = h_ptr[r + 1] - h_ptr[r];
            }
            sp[s + 1] = sp[s] + 32ull * w;
        }
        /* item costs: a header (2 for rows, 3 for a slice), one step per g
         * entries of the group's longest row (the first: rows are longest
         * first) or per entry of the slice, and log2 g steps of the tree */
        for (size_t k = 0; k < ni; ++k) {
            unsigned first, g, tree;
            if (k < it16) {
                first = (unsigned)k, g = 32, tree = 5;
            } else if (k < it4) {
                first = (unsigned)(r32 + 2 * (k - it16)), g = 16, tree = 4;
            } else if (k < itl) {
                first = (unsigned)(r16 + 8 * (k - it4)), g = 4, tree = 2;
            } else {
                cost[k] = 3u + (unsigned)((sp[k - itl + 1] - sp[k - itl]) / 32);
                continue;
            }
            cost[k] = 2u + (wrng[2 * first + 1] - wrng[2 * first] + g - 1) / g + tree;
        }
        rc = hbicg__hyb_plan(ni, cost, hnw, wrow + nw, wrow + nw + hnw + 1);
        if (rc) goto done;
    }
#define HTRY(call)                                                                               \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));          \
            rc = HBICG_E_CUDA;                                                                   \
            goto done;                                                                           \
        }                                                                                        \
    } while (0)
    HTRY(cudaMalloc((void **)&A->d_hsptr, sizeof(unsigned long long) * (ns + 1)));
    HTRY(cudaMalloc((void **)&A->d_hval, sizeof(double) * (sp[ns] + 1)));
    HTRY(cudaMalloc((void **)&A->d_hcol, sizeof(unsigned) * (sp[ns] + 1)));
    HTRY(cudaMalloc((void **)&A->d_srow, srow_bytes));
    HTRY(cudaMalloc((void **)&A->d_wrow, sizeof(unsigned) * plan_words));
    HTRY(cudaMemcpyAsync(A->d_hsptr, sp, sizeof(unsigned long long) * (ns + 1), cudaMemcpyHostToDevice, st));
    if (cap) HTRY(cudaMemcpyAsync(A->d_srow, srow, srow_bytes, cudaMemcpyHostToDevice, st));
    HTRY(cudaMemcpyAsync(A->d_wrow, wrng, sizeof(unsigned) * plan_words, cudaMemcpyHostToDevice, st));
    {
        const int e = hbk_hyb_fill((unsigned)ns, A->d_srow, n, A->d_ptr, A->d_col, A->d_val, A->d_hsptr, A->d_hval,
                                   A->d_hcol, st);
        if (e) HTRY((cudaError_t)e);
    }
    HTRY(cudaStreamSynchronize(st));
#undef HTRY
    A->nslice = (unsigned)ns;
    A->nwrow = (unsigned)nw;
    A->slen_off = cap + 1;
    A->hnw = hnw;
    A->hyb_grid = hgrid;
    A->hrow32 = (unsigned)r32;
    A->hrow16 = (unsigned)r16;
    A->hit16 = (unsigned)it16;
    A->hit4 = (unsigned)it4;
    A->hitl = (unsigned)itl;
done:
    if (rc != HBICG_OK) { /* no half-built form: a later request builds it again */
        cudaStreamSynchronize(st);
        cudaFree(A->d_hsptr);
        cudaFree(A->d_hval);
        cudaFree(A->d_hcol);
        cudaFree(A->d_srow);
        cudaFree(A->d_wrow);
        A->d_hsptr = NULL;
        A->d_hval = NULL;
        A->d_hcol = NULL;
        A->d_srow = NULL;
        A->d_wrow = NULL;
    }
    free(srow);
    free(wkey);
    free(wrng);
    free(cost);
    free(sp);
    return rc;
}

/* point the kernel view at the HYB arrays.  Work items, in order: the long
 * rows above HBK_HYB_L16 entries one each ([0, hrow32), 32 lanes per row),
 * then pairs of rows above HBK_HYB_L4 ([hrow32, hrow16), 16 lanes per row),
 * then groups of 8 rows ([hrow16, nwrow), 4 lanes per row), then the slices. */
static void use_hyb(hbicg_matrix *A) {
    A->k.fmt = HBK_FMT_HYB;
    A->k.sval = A->d_hval;
    A->k.scol = A->d_hcol;
    A->k.sptr = A->d_hsptr;
    A->k.srow = A->d_srow;
    A->k.slen = A->d_srow ? (const unsigned char *)(A->d_srow + A->slen_off) : NULL;
    A->k.wrng = A->d_wrow;
    A->k.wrow = A->d_wrow ? A->d_wrow + 2 * (size_t)A->nwrow : NULL;
    A->k.hwbeg = A->k.wrow ? A->k.wrow + A->nwrow : NULL;
    A->k.hitem = A->k.hwbeg ? A->k.hwbeg + A->hnw + 1 : NULL;
    A->k.hnw = A->hnw;
    A->k.hrow32 = A->hrow32;
    A->k.hrow16 = A->hrow16;
    A->k.hit16 = A->hit16;
    A->k.hit4 = A->hit4;
    A->k.hitl = A->hitl;
    A->k.nslice = A->nslice;
    A->k.nwrow = A->nwrow;
    A->k.grid = A->hyb_grid > 0 ? A->hyb_grid : 1;
}

/* MERGE: rows of at most HBK_MERGE_LONG entries in blocks of consecutive
 * rows with rows + nonzeros <= HBK_MERGE_ITEMS (a block ends where the next
 * row would not fit and before every long row); rows above HBK_MERGE_LONG in
 * a list, longest first (stable), one warp each.  A block is one warp's unit:
 * the device splits it among the lanes along the merge path of row ends and
 * nonzeros, so each lane gets the same number of items whatever the row lengths: for
 * power-law rows this needs no sorting, padding or copy of the values. */
static int build_merge(hbicg_matrix *A, const unsigned *h_ptr, unsigned n) {
    if (!n || A->d_merge) return HBICG_OK;
    size_t nlong = 0, nblk = 0;
    unsigned items = 0;
    int open = 0;
    for (unsigned r = 0; r < n; ++r) {
        const unsigned len = h_ptr[r + 1] - h_ptr[r];
        if (len > HBK_MERGE_LONG) {
            nlong++;
            open = 0;
            continue;
        }
        if (!open || items + len + 1 > HBK_MERGE_ITEMS) {
            nblk++;
            open = 1;
            items = 0;
        }
        items += len + 1;
    }
    const size_t words = 2 * nblk + nlong + 1;
    unsigned *h = malloc(sizeof(unsigned) * words);
    unsigned long long *key = malloc(sizeof(unsigned long long) * (nlong + 1));
    int rc = HBICG_OK;
    if (!h || !key) {
        rc = HBICG_E_NOMEM;
        goto done;
    }
    {
        size_t b = 0, l = 0;
        open = 0;
        items = 0;
        for (unsigned r = 0; r < n; ++r) {
            const unsigned len = h_ptr[r + 1] - h_ptr[r];
            if (len > HBK_MERGE_LONG) {
                /* longest first, then by row */
                key[l++] = ((unsigned long long)(0xFFFFFFFFu - len) << 32) | r;
                if (open) h[2 * b - 1] = r;
                open = 0;
                continue;
            }
            if (!open || items + len + 1 > HBK_MERGE_ITEMS) {
                if (open) h[2 * b - 1] = r;
                h[2 * b] = r;
                b++;
                open = 1;
                items = 0;
            }
            items += len + 1;
        }
        if (open) h[2 * b - 1] = n;
        qsort(key, nlong, sizeof *key, cmp_u64);
        for (size_t i = 0; i < nlong; ++i) h[2 * nblk + i] = (unsigned)(key[i] & 0xFFFFFFFFu);
        h[words - 1] = 0;
    }
    {
        cudaStream_t st = A->ctx->stream;
        cudaError_t e = cudaMalloc((void **)&A->d_merge, sizeof(unsigned) * words);
        if (!e) e = cudaMemcpyAsync(A->d_merge, h, sizeof(unsigned) * words, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaStreamSynchronize(st);
        if (e) {
            set_msg("merge plan: %s", cudaGetErrorString(e));
            rc = e == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;
            cudaFree(A->d_merge);
            A->d_merge = NULL;
            goto done;
        }
    }
    A->nmblk = (unsigned)nblk;
    A->nmlong = (unsigned)nlong;
done:
    free(h);
    free(key);
    return rc;
}

/* point the kernel view at the MERGE plan */
static void use_merge(hbicg_matrix *A) {
    A->k.fmt = HBK_FMT_MERGE;
    A->k.mblk = A->d_merge;
    A->k.nmblk = A->nmblk;
    A->k.mlong = A->d_merge ? A->d_merge + 2 * (size_t)A->nmblk : NULL;
    A->k.nmlong = A->nmlong;
    A->k.grid = hbk_merge_grid(A->nmlong + A->nmblk);
}

/* SELL-32 when every row fits in HBK_SELL_MAX_LEN and padding stays under a
 * third of the nonzeros (rows are short and regular, as in stencils); the CSR
 * row-block path otherwise.  HBICG_SPMV_FORMAT=tile|sell overrides. */
static int build_sell(hbicg_matrix *A, const unsigned *h_ptr, unsigned n, unsigned nnz, int force) {
    cudaStream_t st = A->ctx->stream;
    unsigned maxlen = 0;
    for (unsigned i = 0; i < n; i++)
        if (h_ptr[i + 1] - h_ptr[i] > maxlen) maxlen = h_ptr[i + 1] - h_ptr[i];
    const char *env = force ? "sell" : getenv("HBICG_SPMV_FORMAT");
    int want = maxlen <= HBK_SELL_MAX_LEN;
    if (env && !strcmp(env, "tile")) want = 0;
    if (env && !strcmp(env, "sell")) want = maxlen <= HBK_SELL_MAX_LEN;
    if (!want || !n) return HBICG_OK;
    const unsigned ns = (n + 31) / 32;
    int rc = HBICG_OK;
    unsigned *d_w = NULL, *h_w = malloc(sizeof(unsigned) * ns);
    unsigned long long *h_sp = malloc(sizeof(unsigned long long) * ((size_t)ns + 1));
    if (!h_w || !h_sp) {
        rc = HBICG_E_NOMEM;
        goto out;
    }
    CUDA_GOTO(cudaMalloc((void **)&d_w, sizeof(unsigned) * ns));
    HBK_GOTO(hbk_sell_widths(n, A->d_ptr, d_w, st));
    CUDA_GOTO(cudaMemcpyAsync(h_w, d_w, sizeof(unsigned) * ns, cudaMemcpyDeviceToHost, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
    h_sp[0] = 0;
    for (unsigned i = 0; i < ns; i++) h_sp[i + 1] = h_sp[i] + 32ull * h_w[i];
    const unsigned long long padded = h_sp[ns];
    if (!env && (double)padded > 1.34 * (double)nnz + 4096.0) goto out; /* too much padding: not SELL-32 */
    CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_sptr, sizeof(unsigned long long) * ((size_t)ns + 1), st));
    CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_sval, sizeof(double) * (padded + 1), st));
    CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_scol, sizeof(unsigned) * (padded + 1), st));
    CUDA_GOTO(cudaMemcpyAsync(A->d_sptr, h_sp, sizeof(unsigned long long) * ((size_t)ns + 1), cudaMemcpyHostToDevice,
                              st));
    HBK_GOTO(hbk_sell_fill(n, A->d_ptr, A->d_col, A->d_val, A->d_sptr, A->d_sval, A->d_scol, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
    A->k.fmt = HBK_FMT_SELL;
    A->k.sval = A->d_sval;
    A->k.scol = A->d_scol;
    A->k.sptr = A->d_sptr;
    A->k.sell_len = padded;
    A->diag_state = 0; /* a new SELL-32 layout */
out:
    cudaFree(d_w);
    free(h_w);
    free(h_sp);
    return rc;
}

/* diagonal positions of the SELL-32 form (computed once per layout) */
int hbicg__sell_diag(hbicg_matrix *A) {
    if (A->diag_state) return HBICG_OK;
    cudaStream_t st = A->ctx->stream;
    const unsigned n = A->k.n;
    int *d_missing = NULL, missing = 0;
    int rc = HBICG_OK;
    if (!A->d_sdiag) CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_sdiag, sizeof(unsigned long long) * ((size_t)n + 1), st));
    CUDA_GOTO(cudaMalloc((void **)&d_missing, sizeof(int)));
    CUDA_GOTO(cudaMemsetAsync(d_missing, 0, sizeof(int), st));
    HBK_GOTO(hbk_sell_diag(n, A->d_ptr, A->d_sptr, A->d_scol, A->d_sdiag, d_missing, st));
    CUDA_GOTO(cudaMemcpyAsync(&missing, d_missing, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
    A->diag_state = missing ? 2 : 1;
out: /* d_missing is freed on every path; d_sdiag belongs to the matrix */
    cudaFree(d_missing);
    return rc;
}

/* row blocks of the tile form (hbk_plan_rows) */
static int build_tile_plan(hbicg_matrix *A, const unsigned *h_ptr) {
    cudaStream_t st = A->ctx->stream;
    const unsigned n = A->k.n;
    const unsigned nb = hbk_plan_rows(n, h_ptr, NULL, NULL);
    unsigned *blk = malloc(sizeof(unsigned) * ((size_t)nb + 1));
    unsigned char *kind = malloc((size_t)nb + 1);
    int rc = HBICG_OK;
    if (!blk || !kind) {
        rc = HBICG_E_NOMEM;
    } else {
        hbk_plan_rows(n, h_ptr, blk, kind);
        cudaError_t e = cudaMalloc((void **)&A->d_blk_row, sizeof(unsigned) * ((size_t)nb + 1));
        if (!e) e = cudaMalloc((void **)&A->d_blk_kind, (size_t)nb + 1);
        if (!e) e = cudaMemcpyAsync(A->d_blk_row, blk, sizeof(unsigned) * ((size_t)nb + 1), cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(A->d_blk_kind, kind, (size_t)nb + 1, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaStreamSynchronize(st);
        if (e) {
            set_msg("tile plan: %s", cudaGetErrorString(e));
            rc = HBICG_E_CUDA;
        }
    }
    free(blk);
    free(kind);
    if (rc) return rc;
    A->k.blk_row = A->d_blk_row;
    A->k.blk_kind = A->d_blk_kind;
    A->k.nblk = nb;
    A->k.grid = hbk_spmv_grid(nb);
    return HBICG_OK;
}

static void hbicg_matrix_destroy_unretained(hbicg_matrix *A);

int hbicg_matrix_create(hbicg_context *ctx, unsigned n, unsigned nnz, const unsigned *ptr, const unsigned *col,
                        const double *val, int where, hbicg_matrix **out) {
    hbicg_matrix *A = calloc(1, sizeof *A);
    if (!A) return HBICG_E_NOMEM;
    A->ctx = ctx;
    cudaStream_t st = ctx->stream;
    unsigned *h_ptr = NULL;
    int rc = HBICG_OK;
    if (where == HBICG_DEVICE) {
        A->d_ptr = (unsigned *)ptr;
        A->d_col = (unsigned *)col;
        A->d_val = (double *)val;
        A->owns = 0;
        h_ptr = malloc(sizeof(unsigned) * ((size_t)n + 1));
        if (!h_ptr) {
            rc = HBICG_E_NOMEM;
            goto out;
        }
        CUDA_GOTO(cudaMemcpyAsync(h_ptr, ptr, sizeof(unsigned) * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
        CUDA_GOTO(cudaStreamSynchronize(st));
    } else {
        A->owns = 1;
        A->pooled = 1;
        CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_ptr, sizeof(unsigned) * ((size_t)n + 1), st));
        CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_col, sizeof(unsigned) * ((size_t)nnz + 1), st));
        CUDA_GOTO(hbicg__dev_alloc((void **)&A->d_val, sizeof(double) * ((size_t)nnz + 1), st));
        CUDA_GOTO(cudaMemcpyAsync(A->d_ptr, ptr, sizeof(unsigned) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
        if (nnz) {
            CUDA_GOTO(cudaMemcpyAsync(A->d_col, col, sizeof(unsigned) * (size_t)nnz, cudaMemcpyHostToDevice, st));
            CUDA_GOTO(cudaMemcpyAsync(A->d_val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
        }
        h_ptr = (unsigned *)ptr;
    }
    if (h_ptr[n] != nnz) {
        set_msg("ptr[n] = %u but nnz = %u", h_ptr[n], nnz);
        rc = HBICG_E_ARG;
        goto out;
    }
    A->k.n = n;
    A->k.nnz = nnz;
    A->k.ptr = A->d_ptr;
    A->k.col = A->d_col;
    A->k.val = A->d_val;
    A->k.fmt = HBK_FMT_TILE;
    /* SELL-32 for regular rows, HYB for irregular ones, the tile form on
     * request; the tile form's row plan is built only when it is used */
    rc = build_sell(A, h_ptr, n, nnz, 0);
    const char *env = getenv("HBICG_SPMV_FORMAT");
    if (!rc && A->k.fmt != HBK_FMT_SELL && n && !(env && !strcmp(env, "tile"))) {
        rc = build_hyb(A, h_ptr, n);
        if (!rc) use_hyb(A);
    }
    if (!rc && A->k.fmt == HBK_FMT_TILE) rc = build_tile_plan(A, h_ptr);
out: /* on failure the partial matrix goes, its device arrays with it */
    if (where == HBICG_DEVICE) free(h_ptr);
    if (rc) {
        hbicg_matrix_destroy_unretained(A);
        return rc;
    }
    if (A->k.fmt == HBK_FMT_SELL) A->k.grid = hbk_spmv_grid((n + HBK_THREADS - 1) / HBK_THREADS);
    hbicg__ctx_retain(ctx);
    *out = A;
    return HBICG_OK;
}

int hbicg_matrix_from_coo(hbicg_context *ctx, unsigned n, unsigned nnz, const unsigned *row, const unsigned *col,
                          const double *val, int where, hbicg_matrix **out) {
    if (!ctx || !out || (nnz && (!row || !col || !val))) return HBICG_E_ARG;
    cudaStream_t st = ctx->stream;
    unsigned *d_row = (unsigned *)row, *d_col = (unsigned *)col;
    double *d_val = (double *)val;
    unsigned *ptr = NULL, *colo = NULL;
    double *valo = NULL;
    void *tmp = NULL;
    int *d_err = NULL, h_err = 0, rc = HBICG_OK;
    cudaError_t e = cudaSuccess;
#define FC(call)                                                                 \
    do {                                                                         \
        if ((e = (call)) != cudaSuccess) {                                       \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e)); \
            rc = HBICG_E_CUDA;                                                   \
            goto fail;                                                           \
        }                                                                        \
    } while (0)
    if (where != HBICG_DEVICE) {
        d_row = NULL;
        d_col = NULL;
        d_val = NULL;
        FC(cudaMalloc((void **)&d_row, sizeof(unsigned) * ((size_t)nnz + 1)));
        FC(cudaMalloc((void **)&d_col, sizeof(unsigned) * ((size_t)nnz + 1)));
        FC(cudaMalloc((void **)&d_val, sizeof(double) * ((size_t)nnz + 1)));
        if (nnz) {
            FC(cudaMemcpyAsync(d_row, row, sizeof(unsigned) * (size_t)nnz, cudaMemcpyHostToDevice, st));
            FC(cudaMemcpyAsync(d_col, col, sizeof(unsigned) * (size_t)nnz, cudaMemcpyHostToDevice, st));
            FC(cudaMemcpyAsync(d_val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
        }
    }
    FC(cudaMalloc((void **)&ptr, sizeof(unsigned) * ((size_t)n + 1)));
    FC(cudaMalloc((void **)&colo, sizeof(unsigned) * ((size_t)nnz + 1)));
    FC(cudaMalloc((void **)&valo, sizeof(double) * ((size_t)nnz + 1)));
    FC(cudaMalloc(&tmp, hbk_coo_to_csr_tmp_bytes(nnz)));
    FC(cudaMalloc((void **)&d_err, sizeof(int)));
    FC(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    FC((cudaError_t)hbk_coo_to_csr(n, nnz, d_row, d_col, d_val, ptr, colo, valo, tmp, d_err, st));
    FC(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FC(cudaStreamSynchronize(st));
    if (h_err) {
        set_msg("a row or column index is >= n = %u", n);
        rc = HBICG_E_ARG;
        goto fail;
    }
    cudaFree(tmp);
    cudaFree(d_err);
    tmp = NULL;
    d_err = NULL;
    if (where != HBICG_DEVICE) {
        cudaFree(d_row);
        cudaFree(d_col);
        cudaFree(d_val);
    }
    {
        hbicg_matrix *A = NULL;
        rc = hbicg_matrix_create(ctx, n, nnz, ptr, colo, valo, HBICG_DEVICE, &A);
        if (rc != HBICG_OK) {
            cudaFree(ptr);
            cudaFree(colo);
            cudaFree(valo);
            return rc;
        }
        A->owns = 1;
        *out = A;
    }
    return HBICG_OK;
fail:
    if (where != HBICG_DEVICE) {
        cudaFree(d_row);
        cudaFree(d_col);
        cudaFree(d_val);
    }
    cudaFree(ptr);
    cudaFree(colo);
    cudaFree(valo);
    cudaFree(tmp);
    cudaFree(d_err);
    return rc;
#undef FC
}

int hbicg_matrix_get_csr(const hbicg_matrix *A, unsigned *ptr, unsigned *col, double *val, int where) {
    if (!A) return HBICG_E_ARG;
    cudaStream_t st = A->ctx->stream;
    const enum cudaMemcpyKind kind = where == HBICG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t n = A->k.n, nnz = A->k.nnz;
    if (ptr) CUDA_TRY(cudaMemcpyAsync(ptr, A->d_ptr, sizeof(unsigned) * (n + 1), kind, st));
    if (col && nnz) CUDA_TRY(cudaMemcpyAsync(col, A->d_col, sizeof(unsigned) * nnz, kind, st));
    if (val && nnz) CUDA_TRY(cudaMemcpyAsync(val, A->d_val, sizeof(double) * nnz, kind, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return HBICG_OK;
}

int hbicg_matrix_load_mm(hbicg_context *ctx, const char *path, int expand_symmetric, hbicg_matrix **out) {
    hbicg_coo c;
    int rc = hbicg_mm_read(path, expand_symmetric, 0, &c);
    if (rc != HBICG_OK) return rc;
    if (c.rows != c.cols) {
        set_msg("%s is %u x %u, not square", path, c.rows, c.cols);
        hbicg_coo_free(&c);
        return HBICG_E_NOT_SQUARE;
    }
    if (c.nnz > 0xFFFFFFFFull) {
        set_msg("%s has %llu entries; at most 2^32 - 1 are supported", path, c.nnz);
        hbicg_coo_free(&c);
        return HBICG_E_ARG;
    }
    rc = hbicg_matrix_from_coo(ctx, c.rows, (unsigned)c.nnz, c.row, c.col, c.val, HBICG_HOST, out);
    hbicg_coo_free(&c);
    return rc;
}

/* frees a matrix whose creation failed before it took its context reference */
/* the matrix's device arrays: the CSR copy (when it owns one), the SELL-32
 * form and the diagonal positions from the pool, the rest plain */
static void free_device_arrays(hbicg_matrix *A) {
    cudaStream_t st = A->ctx->stream;
    cudaStreamSynchronize(st);
    if (A->owns) {
        if (A->pooled) {
            hbicg__dev_free(A->d_ptr, st);
            hbicg__dev_free(A->d_col, st);
            hbicg__dev_free(A->d_val, st);
        } else {
            cudaFree(A->d_ptr);
            cudaFree(A->d_col);
            cudaFree(A->d_val);
        }
    }
    cudaFree(A->d_blk_row);
    cudaFree(A->d_blk_kind);
    hbicg__dev_free(A->d_sval, st);
    hbicg__dev_free(A->d_scol, st);
    hbicg__dev_free(A->d_sptr, st);
    cudaFree(A->d_hval);
    cudaFree(A->d_hcol);
    cudaFree(A->d_hsptr);
    cudaFree(A->d_srow);
    cudaFree(A->d_wrow);
    hbicg__dev_free(A->d_sdiag, st);
    cudaFree(A->d_merge);
    cudaStreamSynchronize(st);
}

static void hbicg_matrix_destroy_unretained(hbicg_matrix *A) {
    free_device_arrays(A);
    free(A);
}

void hbicg_matrix_destroy(hbicg_matrix *A) {
    if (!A) return;
    free_device_arrays(A);
    hbicg_context *ctx = A->ctx;
    free(A);
    hbicg__ctx_release(ctx);
}

const hbk_matrix *hbicg__matrix_kernel_view(const hbicg_matrix *A) { return &A->k; }
hbicg_context *hbicg__matrix_context(const hbicg_matrix *A) { return A->ctx; }

unsigned hbicg_matrix_rows(const hbicg_matrix *A) { return A->k.n; }
unsigned long long hbicg_matrix_nnz(const hbicg_matrix *A) { return A->k.nnz; }

int hbicg_matrix_spmv(hbicg_matrix *A, const double *x, double *y, double sigma, int where) {
    cudaStream_t st = A->ctx->stream;
    const unsigned n = A->k.n;
    if (where == HBICG_DEVICE) {
        HBK_TRY(hbk_spmv(&A->k, x, y, sigma, sigma != 0.0, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return HBICG_OK;
    }
    double *dx = NULL, *dy = NULL;
    CUDA_TRY(cudaMalloc((void **)&dx, sizeof(double) * ((size_t)n + 1)));
    CUDA_TRY(cudaMalloc((void **)&dy, sizeof(double) * ((size_t)n + 1)));
    CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    HBK_TRY(hbk_spmv(&A->k, dx, dy, sigma, sigma != 0.0, st));
    CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(dx);
    cudaFree(dy);
    return HBICG_OK;
}

int hbicg_matrix_time_spmv(hbicg_matrix *A, const double *x, double *y, double sigma, int iters, double *ms) {
    cudaStream_t st = A->ctx->stream;
    if (iters < 1) iters = 1;
    HBK_TRY(hbk_spmv(&A->k, x, y, sigma, sigma != 0.0, st)); /* warm */
    CUDA_TRY(cudaEventRecord(A->ctx->ev0, st));
    for (int i = 0; i < iters; i++) HBK_TRY(hbk_spmv(&A->k, x, y, sigma, sigma != 0.0, st));
    CUDA_TRY(cudaEventRecord(A->ctx->ev1, st));
    CUDA_TRY(cudaEventSynchronize(A->ctx->ev1));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, A->ctx->ev0, A->ctx->ev1));
    *ms = (double)t / iters;
    return HBICG_OK;
}

int hbicg_matrix_format(const hbicg_matrix *A) {
    switch (A->k.fmt) {
    case HBK_FMT_SELL: return HBICG_SPMV_SELL;
    case HBK_FMT_HYB: return HBICG_SPMV_HYB;
    case HBK_FMT_MERGE: return HBICG_SPMV_MERGE;
    default: return HBICG_SPMV_TILE;
    }
}

static unsigned *host_ptr_copy(hbicg_matrix *A) {
    const size_t n = A->k.n;
    unsigned *hp = malloc(sizeof(unsigned) * (n + 1));
    if (!hp) return NULL;
    if (cudaMemcpy(hp, A->d_ptr, sizeof(unsigned) * (n + 1), cudaMemcpyDeviceToHost) != cudaSuccess) {
        free(hp);
        return NULL;
    }
    return hp;
}

int hbicg_matrix_set_format(hbicg_matrix *A, int fmt) {
    if (!A || (fmt != HBICG_SPMV_TILE && fmt != HBICG_SPMV_SELL && fmt != HBICG_SPMV_HYB && fmt != HBICG_SPMV_MERGE))
        return HBICG_E_ARG;
    if (fmt == HBICG_SPMV_MERGE) {
        if (!A->d_merge && A->k.n) {
            unsigned *hp = host_ptr_copy(A);
            if (!hp) return HBICG_E_NOMEM;
            int rc = build_merge(A, hp, A->k.n);
            free(hp);
            if (rc) return rc;
        }
        use_merge(A);
        return HBICG_OK;
    }
    if (fmt == HBICG_SPMV_TILE) {
        if (!A->d_blk_row) {
            unsigned *hp = host_ptr_copy(A);
            if (!hp) return HBICG_E_NOMEM;
            int rc = build_tile_plan(A, hp);
            free(hp);
            if (rc) return rc;
        }
        A->k.fmt = HBK_FMT_TILE;
        A->k.grid = hbk_spmv_grid(A->k.nblk);
        return HBICG_OK;
    }
    if (fmt == HBICG_SPMV_HYB) {
        if (!A->d_hval && A->k.n) {
            unsigned *hp = host_ptr_copy(A);
            if (!hp) return HBICG_E_NOMEM;
            int rc = build_hyb(A, hp, A->k.n);
            free(hp);
            if (rc) return rc;
        }
        use_hyb(A);
        return HBICG_OK;
    }
    if (!A->d_sval) {
        unsigned *hp = host_ptr_copy(A);
        if (!hp) return HBICG_E_NOMEM;
        int rc = build_sell(A, hp, A->k.n, A->k.nnz, 1);
        free(hp);
        if (rc) return rc;
        if (!A->d_sval) {
            set_msg("a row is longer than %d entries: no SELL-32 form", HBK_SELL_MAX_LEN);
            return HBICG_E_ARG;
        }
    }
    A->k.fmt = HBK_FMT_SELL;
    A->k.sval = A->d_sval;
    A->k.scol = A->d_scol;
    A->k.sptr = A->d_sptr;
    A->k.grid = hbk_spmv_grid((A->k.n + HBK_THREADS - 1) / HBK_THREADS);
    return HBICG_OK;
}

/* Signature of a sparsity pattern for the autotune cache: log2 of n, the
 * longest row, and the share of rows in each power-of-two row-length class
 * (0, 1, 2-3, 4-7, ..., >= 8192), in sixteenths. */
static void pattern_signature(const unsigned *hp, unsigned n, char *key, size_t cap) {
    unsigned long long cls[15] = {0};
    unsigned maxlen = 0;
    for (unsigned i = 0; i < n; i++) {
        const unsigned len = hp[i + 1] - hp[i];
        if (len > maxlen) maxlen = len;
        int c = 0;
        for (unsigned v = len; v && c < 14; v >>= 1) ++c;
        cls[c]++;
    }
    int lg = 0;
    for (unsigned v = n; v > 1; v >>= 1) ++lg;
    int o = snprintf(key, cap, "n2^%d:max%u:", lg, maxlen);
    for (int c = 0; c < 15 && o < (int)cap; ++c) {
        const unsigned q = n ? (unsigned)((16ull * cls[c] + n / 2) / n) : 0u;
        o += snprintf(key + o, cap - (size_t)o, "%x", q > 15 ? 15u : q);
    }
}

static pthread_mutex_t g_tune_lock = PTHREAD_MUTEX_INITIALIZER;

/* cached choice for key: 0 tile, 1 sell, 2 hyb, -1 none */
static int tune_lookup(const char *path, const char *key, double *tile_ms, double *sell_ms) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char line[512], k[256], fmt[16];
    int found = -1;
    while (fgets(line, sizeof line, f)) {
        double t, sl;
        if (line[0] == '#') continue;
        if (sscanf(line, "%255s %15s %lf %lf", k, fmt, &t, &sl) == 4 && !strcmp(k, key)) {
            found = !strcmp(fmt, "sell") ? 1 : !strcmp(fmt, "hyb") ? 2 : !strcmp(fmt, "merge") ? 3 : 0;
            *tile_ms = t;
            *sell_ms = sl;
        }
    }
    fclose(f);
    return found;
}

int hbicg_matrix_autotune(hbicg_matrix *A, const char *cache_path, int *chosen, double *tile_ms, double *sell_ms) {
    if (!A) return HBICG_E_ARG;
    unsigned *hp = host_ptr_copy(A);
    if (!hp) return HBICG_E_NOMEM;
    char key[256];
    pattern_signature(hp, A->k.n, key, sizeof key);
    free(hp);
    double t_tile = -1.0, t_sell = -1.0;
    int pick = -1;
    if (cache_path && *cache_path) {
        pthread_mutex_lock(&g_tune_lock);
        pick = tune_lookup(cache_path, key, &t_tile, &t_sell);
        pthread_mutex_unlock(&g_tune_lock);
    }
    if (pick < 0) {
        /* time both forms of y = A x (10 launches each after a warm-up) */
        const size_t n = A->k.n ? A->k.n : 1;
        double *x = NULL, *y = NULL;
        cudaError_t e = cudaMalloc((void **)&x, sizeof(double) * n);
        if (!e) e = cudaMalloc((void **)&y, sizeof(double) * n);
        if (!e) e = cudaMemsetAsync(x, 0, sizeof(double) * n, A->ctx->stream);
        if (e) {
            cudaFree(x);
            cudaFree(y);
            set_msg("autotune buffers: %s", cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;
        }
        int rc = hbicg_matrix_set_format(A, HBICG_SPMV_TILE);
        if (!rc) rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_tile);
        double t_s = -1.0, t_h = -1.0, t_m = -1.0;
        if (!rc && hbicg_matrix_set_format(A, HBICG_SPMV_SELL) == HBICG_OK)
            rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_s);
        if (!rc && hbicg_matrix_set_format(A, HBICG_SPMV_HYB) == HBICG_OK)
            rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_h);
        if (!rc && hbicg_matrix_set_format(A, HBICG_SPMV_MERGE) == HBICG_OK)
            rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_m);
        cudaFree(x);
        cudaFree(y);
        if (rc) return rc;
        pick = 0;
        double best = t_tile;
        const double tt[4] = {t_tile, t_s, t_h, t_m};
        for (int f = 1; f < 4; ++f)
            if (tt[f] >= 0.0 && tt[f] < best) {
                pick = f;
                best = tt[f];
            }
        /* the packed form's time: the fastest of SELL-32, HYB and MERGE */
        t_sell = -1.0;
        for (int f = 1; f < 4; ++f)
            if (tt[f] >= 0.0 && (t_sell < 0.0 || tt[f] < t_sell)) t_sell = tt[f];
        if (cache_path && *cache_path) {
            char line[512];
            static const char *names[4] = {"tile", "sell", "hyb", "merge"};
            const int len = snprintf(line, sizeof line, "%s %s %.6f %.6f\n", key, names[pick], t_tile, t_sell);
            pthread_mutex_lock(&g_tune_lock);
            const int fd = open(cache_path, O_WRONLY | O_CREAT | O_APPEND, 0644);
            if (fd >= 0) {
                struct stat sb;
                if (fstat(fd, &sb) == 0 && sb.st_size == 0) {
                    static const char head[] = "# hbicg autotune cache v1: signature format tile_ms sell_ms\n";
                    if (write(fd, head, sizeof head - 1) < 0) { /* best effort */
                    }
                }
                if (write(fd, line, (size_t)len) < 0) { /* a cache that cannot be written is only slower */
                }
                close(fd);
            }
            pthread_mutex_unlock(&g_tune_lock);
        }
    }
    static const int fmts[4] = {HBICG_SPMV_TILE, HBICG_SPMV_SELL, HBICG_SPMV_HYB, HBICG_SPMV_MERGE};
    int rc = hbicg_matrix_set_format(A, fmts[pick]);
    if (rc) return rc;
    /* give the memory of the forms not chosen back; the kernel view keeps
     * only pointers into the chosen form (SELL-32 and HYB share its
     * sval/scol/sptr fields, so only pointers to the freed arrays are cleared) */
    if (pick != 2 && A->d_hval) { /* the HYB copy is not used */
        cudaStreamSynchronize(A->ctx->stream);
        if (A->k.sval == A->d_hval) {
            A->k.sval = NULL;
            A->k.scol = NULL;
            A->k.sptr = NULL;
        }
        cudaFree(A->d_hval);
        cudaFree(A->d_hcol);
        cudaFree(A->d_hsptr);
        cudaFree(A->d_srow);
        cudaFree(A->d_wrow);
        A->d_hval = NULL;
        A->d_hcol = NULL;
        A->d_hsptr = NULL;
        A->d_srow = NULL;
        A->d_wrow = NULL;
        A->k.srow = NULL;
        A->k.slen = NULL;
        A->k.wrow = NULL;
        A->k.wrng = NULL;
        A->k.hwbeg = NULL;
        A->k.hitem = NULL;
        A->k.hnw = 0;
        A->k.hitl = 0;
        A->k.nslice = 0;
        A->k.nwrow = 0;
    }
    if (pick != 1 && A->d_sval) { /* the SELL copy is not used */
        cudaStreamSynchronize(A->ctx->stream);
        if (A->k.sval == A->d_sval) {
            A->k.sval = NULL;
            A->k.scol = NULL;
            A->k.sptr = NULL;
        }
        hbicg__dev_free(A->d_sval, A->ctx->stream);
        hbicg__dev_free(A->d_scol, A->ctx->stream);
        hbicg__dev_free(A->d_sptr, A->ctx->stream);
        hbicg__dev_free(A->d_sdiag, A->ctx->stream); /* positions in the SELL-32 arrays */
        cudaStreamSynchronize(A->ctx->stream);
        A->d_sval = NULL;
        A->d_scol = NULL;
        A->d_sptr = NULL;
        A->d_sdiag = NULL;
        A->diag_state = 0;
    }
    if (pick != 3 && A->d_merge) { /* the MERGE plan is not used */
        cudaStreamSynchronize(A->ctx->stream);
        cudaFree(A->d_merge);
        A->d_merge = NULL;
        A->k.mblk = NULL;
        A->k.mlong = NULL;
        A->k.nmblk = 0;
        A->k.nmlong = 0;
    }
    if (chosen) *chosen = fmts[pick];
    if (tile_ms) *tile_ms = t_tile;
    if (sell_ms) *sell_ms = t_sell;
    return HBICG_OK;
}

/* Host-pointer product used by the matrix.h entry points: y (+)= A x with A
 * rows x cols.  Runs the CSR SpMV kernel on a process-wide context. */
static hbicg_context *g_host_ctx = NULL;
static pthread_mutex_t g_host_ctx_lock = PTHREAD_MUTEX_INITIALIZER;

int hbicg__host_spmv(unsigned rows, unsigned cols, unsigned nnz, const unsigned *ptr, const unsigned *col,
                     const double *val, const double *x, double *y, int accumulate) {
    if (!rows) return HBICG_OK;
    pthread_mutex_lock(&g_host_ctx_lock); /* created once, whichever thread calls first */
    int crc = g_host_ctx ? HBICG_OK : hbicg_context_create(&g_host_ctx);
    pthread_mutex_unlock(&g_host_ctx_lock);
    if (crc) return crc;
    hbicg_matrix *A = NULL;
    int rc = hbicg_matrix_create(g_host_ctx, rows, nnz, ptr, col, val, HBICG_HOST, &A);
    if (rc) return rc;
    cudaStream_t st = g_host_ctx->stream;
    double *dx = NULL, *dy = NULL;
    CUDA_GOTO(cudaMalloc((void **)&dx, sizeof(double) * ((size_t)cols + 1)));
    CUDA_GOTO(cudaMalloc((void **)&dy, sizeof(double) * ((size_t)rows + 1)));
    if (cols) CUDA_GOTO(cudaMemcpyAsync(dx, x, sizeof(double) * cols, cudaMemcpyHostToDevice, st));
    if (accumulate) {
        CUDA_GOTO(cudaMemcpyAsync(dy, y, sizeof(double) * rows, cudaMemcpyHostToDevice, st));
        HBK_GOTO(hbk_spmv_accumulate(&A->k, dx, dy, st));
    } else {
        HBK_GOTO(hbk_spmv(&A->k, dx, dy, 0.0, 0, st));
    }
    CUDA_GOTO(cudaMemcpyAsync(y, dy, sizeof(double) * rows, cudaMemcpyDeviceToHost, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
out:
    cudaFree(dx);
    cudaFree(dy);
    hbicg_matrix_destroy(A);
    return rc;
}
