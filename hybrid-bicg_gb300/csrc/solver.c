/* Host driver of the GB300 shifted BiCGStab solver (C11 + CUDA runtime).
 *
 * Owns the device workspace, uploads inputs, runs one of the two iteration
 * forms and returns results through the reference's entry points
 * (src/solver.h:33-35) and the extended API (include/hbicg.h):
 *   plain  one kernel per step of the reference's iteration; dot products come
 *          back to the host, which keeps the scalars, runs the shift
 *          recurrences, the convergence test and the seed switch exactly as
 *          src/solver_dynamic.c:147-381 does (the per-kernel form);
 *   fused  five to seven kernels per iteration with every scalar on the device
 *          (hbk_fused_iteration); iterations are captured in CUDA graphs and
 *          the host only polls a finished flag between graph launches.
 * In the fused form the shifts are either updated every iteration by one
 * multi-shift kernel (incremental) or kept as coefficient vectors over the
 * seed's Krylov basis and formed once at the end by an FP64 GEMM-like kernel
 * (deferred), which cuts the FP64 work per shift per iteration by three.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fcntl.h>
#include <pthread.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "hbicg.h"
#include "hbk.h"
#include "solver.h"

/* ------------------------------------------------------------------------ */
static _Thread_local char g_msg[512];

static void set_msg(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
}

const char *hbicg_last_message(void) { return g_msg; }

void hbicg__set_message(const char *msg) { set_msg("%s", msg); }

const char *hbicg_status_string(int s) {
    switch (s) {
    case HBICG_OK: return "ok";
    case HBICG_E_NOT_SQUARE: return "matrix is not square";
    case HBICG_E_NO_DIAG: return "diagonal entry missing";
    case HBICG_E_BREAKDOWN: return "breakdown (zero or non-finite recurrence scalar)";
    case HBICG_E_MAXITER: return "maximum iterations reached";
    case HBICG_E_CUDA: return "CUDA error";
    case HBICG_E_TIMEOUT: return "timeout";
    case HBICG_E_ARG: return "invalid argument";
    case HBICG_E_NOMEM: return "out of device memory";
    case HBICG_E_IO: return "I/O error";
    default: return "unknown status";
    }
}

#define CUDA_TRY(call)                                                                                   \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));                  \
            return e_ == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;                       \
        }                                                                                                \
    } while (0)

#define HBK_TRY(call)                                                                                    \
    do {                                                                                                 \
        int e_ = (call);                                                                                 \
        if (e_) {                                                                                        \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, hbk_error_string(e_));                    \
            return HBICG_E_CUDA;                                                                         \
        }                                                                                                \
    } while (0)

/* the same two checks for functions that own host or device scratch: set rc
 * and leave through their `out:` cleanup */
#define CUDA_GOTO(call)                                                                                  \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));                  \
            rc = e_ == cudaErrorMemoryAllocation ? HBICG_E_NOMEM : HBICG_E_CUDA;                         \
            goto out;                                                                                    \
        }                                                                                                \
    } while (0)
#define HBK_GOTO(call)                                                                                   \
    do {                                                                                                 \
        int e_ = (call);                                                                                 \
        if (e_) {                                                                                        \
            set_msg("%s:%d %s: %s", __FILE__, __LINE__, #call, hbk_error_string(e_));                    \
            rc = HBICG_E_CUDA;                                                                           \
            goto out;                                                                                    \
        }                                                                                                \
    } while (0)

static size_t ld_of(unsigned n) { return ((size_t)n + 31) / 32 * 32; }

void hbicg_params_default(hbicg_params *p) {
    memset(p, 0, sizeof *p);
    p->tol = EPS;
    p->max_iter = MAX_ITER;
    p->switching = 1;
    p->form = HBICG_FORM_FUSED;
    p->shift_mode = HBICG_SHIFTS_AUTO;
    p->use_graph = 1;
    p->graph_chunk = 0;
    p->basis_mem_frac = 0.6;
    p->true_residuals = 0;
    p->basis_block = 0;
    p->flush_mode = HBICG_FLUSH_AUTO;
    p->refine = 1;
}

/* ------------------------------------------------------------------------ */
struct hbicg_context {
    cudaStream_t stream;
    cudaStream_t cstream;  /* copies of finished solutions to the host during a solve */
    cudaEvent_t ev0, ev1, evf0, evf1, cev;
    hbk_scalars *h_sc; /* pinned */
    double *h_dbl;     /* pinned scratch */
    int refs;          /* the caller's handle + one per live matrix or solver */
};

static void ctx_retain(hbicg_context *c) { __atomic_add_fetch(&c->refs, 1, __ATOMIC_RELAXED); }
static void ctx_free(hbicg_context *c);
/* the context is freed when its handle and every matrix and solver made on it
 * are gone, in whatever order a caller (or a garbage collector) destroys them */
static void ctx_release(hbicg_context *c) {
    if (__atomic_sub_fetch(&c->refs, 1, __ATOMIC_ACQ_REL) == 0) ctx_free(c);
}

int hbicg_context_create(hbicg_context **out) {
    hbicg_context *c = calloc(1, sizeof *c);
    if (!c) return HBICG_E_NOMEM;
    c->refs = 1;
    CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&c->cev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreate(&c->ev0));
    CUDA_TRY(cudaEventCreate(&c->ev1));
    CUDA_TRY(cudaEventCreate(&c->evf0));
    CUDA_TRY(cudaEventCreate(&c->evf1));
    CUDA_TRY(cudaMallocHost((void **)&c->h_sc, sizeof(hbk_scalars)));
    CUDA_TRY(cudaMallocHost((void **)&c->h_dbl, sizeof(double) * 64));
    *out = c;
    return HBICG_OK;
}

void hbicg_context_destroy(hbicg_context *c) {
    if (c) ctx_release(c);
}

static void ctx_free(hbicg_context *c) {
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->cstream);
    cudaStreamDestroy(c->cstream);
    cudaEventDestroy(c->cev);
    cudaFreeHost(c->h_sc);
    cudaFreeHost(c->h_dbl);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    cudaEventDestroy(c->evf0);
    cudaEventDestroy(c->evf1);
    cudaStreamDestroy(c->stream);
    free(c);
}

void *hbicg_context_stream(hbicg_context *c) { return (void *)c->stream; }

/* ------------------------------------------------------------------------ */
struct hbicg_matrix {
    hbicg_context *ctx;
    hbk_matrix k;
    unsigned *d_ptr, *d_col;
    double *d_val;
    int owns;
    unsigned *d_blk_row;
    unsigned char *d_blk_kind;
    double *d_sval;
    unsigned *d_scol;
    unsigned long long *d_sptr;
    /* positions of the diagonal entries in the SELL-32 arrays (for folding a
     * shift into the diagonal); diag_state: 0 not computed, 1 ok, 2 a row has
     * no stored diagonal */
    unsigned long long *d_sdiag;
    int diag_state;
    /* HYB form (hbk.h HBK_FMT_HYB) */
    double *d_hval;
    unsigned *d_hcol, *d_srow, *d_wrow; /* d_srow: lane -> row map, then the lanes' row lengths (bytes) */
    size_t slen_off;                    /* entries of the map before the lengths */
    unsigned long long *d_hsptr;
    unsigned nslice, nwrow;
};

static int cmp_u64(const void *a, const void *b) {
    const unsigned long long x = *(const unsigned long long *)a, y = *(const unsigned long long *)b;
    return x < y ? -1 : x > y;
}

/* HYB: rows of at most HBK_HYB_SHORT entries in SELL-32 slices, sorted by
 * length (longest first, stable) inside windows of HBK_HYB_WINDOW consecutive
 * rows, so that the 32 rows of a slice have similar lengths and the rows a
 * warp writes stay inside one window; each window's list is padded to whole
 * slices with empty lanes.  Longer rows go to a list, longest first, one warp
 * each.  For power-law row lengths (most rows short, a few thousands long),
 * where a thread per row leaves most lanes of a warp idle.  The lengths of the
 * slice rows are kept as bytes after the lane -> row map, so that a warp reads
 * its 32 lengths in one line instead of 64 scattered row pointers. */
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
    unsigned *wrow = malloc(sizeof(unsigned) * (nw + 1));
    unsigned long long *sp = malloc(sizeof(unsigned long long) * (ns + 1));
    int rc = HBICG_OK;
    if (!srow || !wkey || !wrow || !sp) {
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
        for (size_t i = 0; i < nw; ++i) wrow[i] = (unsigned)(wkey[i] & 0xFFFFFFFFu);
        sp[0] = 0;
        for (size_t s = 0; s < ns; ++s) {
            unsigned w = 0;
            for (int l = 0; l < 32; ++l) {
                const unsigned r = srow[32 * s + l];
                if (r < n && h_ptr[r + 1] - h_ptr[r] > w) w = h_ptr[r + 1] - h_ptr[r];
            }
            sp[s + 1] = sp[s] + 32ull * w;
        }
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
    HTRY(cudaMalloc((void **)&A->d_wrow, sizeof(unsigned) * (nw + 1)));
    HTRY(cudaMemcpyAsync(A->d_hsptr, sp, sizeof(unsigned long long) * (ns + 1), cudaMemcpyHostToDevice, st));
    if (cap) HTRY(cudaMemcpyAsync(A->d_srow, srow, srow_bytes, cudaMemcpyHostToDevice, st));
    if (nw) HTRY(cudaMemcpyAsync(A->d_wrow, wrow, sizeof(unsigned) * nw, cudaMemcpyHostToDevice, st));
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
done:
    free(srow);
    free(wkey);
    free(wrow);
    free(sp);
    return rc;
}

/* point the kernel view at the HYB arrays */
static void use_hyb(hbicg_matrix *A) {
    A->k.fmt = HBK_FMT_HYB;
    A->k.sval = A->d_hval;
    A->k.scol = A->d_hcol;
    A->k.sptr = A->d_hsptr;
    A->k.srow = A->d_srow;
    A->k.slen = A->d_srow ? (const unsigned char *)(A->d_srow + A->slen_off) : NULL;
    A->k.wrow = A->d_wrow;
    A->k.nslice = A->nslice;
    A->k.nwrow = A->nwrow;
    A->k.grid = hbk_spmv_grid((A->k.n + HBK_THREADS - 1) / HBK_THREADS);
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
    CUDA_GOTO(cudaMalloc((void **)&A->d_sptr, sizeof(unsigned long long) * ((size_t)ns + 1)));
    CUDA_GOTO(cudaMalloc((void **)&A->d_sval, sizeof(double) * (padded + 1)));
    CUDA_GOTO(cudaMalloc((void **)&A->d_scol, sizeof(unsigned) * (padded + 1)));
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
static int sell_diag(hbicg_matrix *A) {
    if (A->diag_state) return HBICG_OK;
    cudaStream_t st = A->ctx->stream;
    const unsigned n = A->k.n;
    int *d_missing = NULL, missing = 0;
    if (!A->d_sdiag) CUDA_TRY(cudaMalloc((void **)&A->d_sdiag, sizeof(unsigned long long) * ((size_t)n + 1)));
    CUDA_TRY(cudaMalloc((void **)&d_missing, sizeof(int)));
    CUDA_TRY(cudaMemsetAsync(d_missing, 0, sizeof(int), st));
    int e = hbk_sell_diag(n, A->d_ptr, A->d_sptr, A->d_scol, A->d_sdiag, d_missing, st);
    if (!e) e = (int)cudaMemcpyAsync(&missing, d_missing, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = (int)cudaStreamSynchronize(st);
    cudaFree(d_missing);
    if (e) {
        set_msg("diagonal positions: %s", cudaGetErrorString((cudaError_t)e));
        return HBICG_E_CUDA;
    }
    A->diag_state = missing ? 2 : 1;
    return HBICG_OK;
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
    if (where == HBICG_DEVICE) {
        A->d_ptr = (unsigned *)ptr;
        A->d_col = (unsigned *)col;
        A->d_val = (double *)val;
        A->owns = 0;
        h_ptr = malloc(sizeof(unsigned) * ((size_t)n + 1));
        if (!h_ptr) return HBICG_E_NOMEM;
        CUDA_TRY(cudaMemcpyAsync(h_ptr, ptr, sizeof(unsigned) * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    } else {
        A->owns = 1;
        CUDA_TRY(cudaMalloc((void **)&A->d_ptr, sizeof(unsigned) * ((size_t)n + 1)));
        CUDA_TRY(cudaMalloc((void **)&A->d_col, sizeof(unsigned) * ((size_t)nnz + 1)));
        CUDA_TRY(cudaMalloc((void **)&A->d_val, sizeof(double) * ((size_t)nnz + 1)));
        CUDA_TRY(cudaMemcpyAsync(A->d_ptr, ptr, sizeof(unsigned) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
        if (nnz) {
            CUDA_TRY(cudaMemcpyAsync(A->d_col, col, sizeof(unsigned) * (size_t)nnz, cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(A->d_val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
        }
        h_ptr = (unsigned *)ptr;
    }
    if (h_ptr[n] != nnz) {
        set_msg("ptr[n] = %u but nnz = %u", h_ptr[n], nnz);
        if (where == HBICG_DEVICE) free(h_ptr);
        free(A);
        return HBICG_E_ARG;
    }
    A->k.n = n;
    A->k.nnz = nnz;
    A->k.ptr = A->d_ptr;
    A->k.col = A->d_col;
    A->k.val = A->d_val;
    A->k.fmt = HBK_FMT_TILE;
    /* SELL-32 for regular rows, HYB for irregular ones, the tile form on
     * request; the tile form's row plan is built only when it is used */
    int rc = build_sell(A, h_ptr, n, nnz, 0);
    const char *env = getenv("HBICG_SPMV_FORMAT");
    if (!rc && A->k.fmt != HBK_FMT_SELL && n && !(env && !strcmp(env, "tile"))) {
        rc = build_hyb(A, h_ptr, n);
        if (!rc) use_hyb(A);
    }
    if (!rc && A->k.fmt == HBK_FMT_TILE) rc = build_tile_plan(A, h_ptr);
    if (where == HBICG_DEVICE) free(h_ptr);
    if (rc) {
        hbicg_matrix_destroy_unretained(A);
        return rc;
    }
    if (A->k.fmt == HBK_FMT_SELL) A->k.grid = hbk_spmv_grid((n + HBK_THREADS - 1) / HBK_THREADS);
    ctx_retain(ctx);
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
static void hbicg_matrix_destroy_unretained(hbicg_matrix *A) {
    cudaStreamSynchronize(A->ctx->stream);
    if (A->owns) {
        cudaFree(A->d_ptr);
        cudaFree(A->d_col);
        cudaFree(A->d_val);
    }
    cudaFree(A->d_blk_row);
    cudaFree(A->d_blk_kind);
    cudaFree(A->d_sval);
    cudaFree(A->d_scol);
    cudaFree(A->d_sptr);
    cudaFree(A->d_hval);
    cudaFree(A->d_hcol);
    cudaFree(A->d_hsptr);
    cudaFree(A->d_srow);
    cudaFree(A->d_wrow);
    cudaFree(A->d_sdiag);
    free(A);
}

void hbicg_matrix_destroy(hbicg_matrix *A) {
    if (!A) return;
    cudaStreamSynchronize(A->ctx->stream);
    if (A->owns) {
        cudaFree(A->d_ptr);
        cudaFree(A->d_col);
        cudaFree(A->d_val);
    }
    cudaFree(A->d_blk_row);
    cudaFree(A->d_blk_kind);
    if (A->d_sval) cudaFree(A->d_sval);
    if (A->d_scol) cudaFree(A->d_scol);
    if (A->d_sptr) cudaFree(A->d_sptr);
    cudaFree(A->d_hval);
    cudaFree(A->d_hcol);
    cudaFree(A->d_hsptr);
    cudaFree(A->d_srow);
    cudaFree(A->d_wrow);
    cudaFree(A->d_sdiag);
    hbicg_context *ctx = A->ctx;
    free(A);
    ctx_release(ctx);
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
    return A->k.fmt == HBK_FMT_SELL ? HBICG_SPMV_SELL : A->k.fmt == HBK_FMT_HYB ? HBICG_SPMV_HYB : HBICG_SPMV_TILE;
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
    if (!A || (fmt != HBICG_SPMV_TILE && fmt != HBICG_SPMV_SELL && fmt != HBICG_SPMV_HYB)) return HBICG_E_ARG;
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
            found = !strcmp(fmt, "sell") ? 1 : !strcmp(fmt, "hyb") ? 2 : 0;
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
        double t_s = -1.0, t_h = -1.0;
        if (!rc && hbicg_matrix_set_format(A, HBICG_SPMV_SELL) == HBICG_OK)
            rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_s);
        if (!rc && hbicg_matrix_set_format(A, HBICG_SPMV_HYB) == HBICG_OK)
            rc = hbicg_matrix_time_spmv(A, x, y, 0.0, 10, &t_h);
        cudaFree(x);
        cudaFree(y);
        if (rc) return rc;
        pick = 0;
        double best = t_tile;
        if (t_s >= 0.0 && t_s < best) {
            pick = 1;
            best = t_s;
        }
        if (t_h >= 0.0 && t_h < best) pick = 2;
        /* the packed form's time: SELL-32 where it exists and was not beaten by HYB */
        t_sell = pick == 2 || t_s < 0.0 ? t_h : t_s;
        if (cache_path && *cache_path) {
            char line[512];
            static const char *names[3] = {"tile", "sell", "hyb"};
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
    int rc = hbicg_matrix_set_format(A, pick == 1 ? HBICG_SPMV_SELL : pick == 2 ? HBICG_SPMV_HYB : HBICG_SPMV_TILE);
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
        cudaFree(A->d_sval);
        cudaFree(A->d_scol);
        cudaFree(A->d_sptr);
        A->d_sval = NULL;
        A->d_scol = NULL;
        A->d_sptr = NULL;
    }
    if (chosen) *chosen = pick == 1 ? HBICG_SPMV_SELL : pick == 2 ? HBICG_SPMV_HYB : HBICG_SPMV_TILE;
    if (tile_ms) *tile_ms = t_tile;
    if (sell_ms) *sell_ms = t_sell;
    return HBICG_OK;
}

/* Host-pointer product used by the matrix.h entry points: y (+)= A x with A
 * rows x cols.  Runs the CSR SpMV kernel on a process-wide context. */
static hbicg_context *g_host_ctx = NULL;

int hbicg__host_spmv(unsigned rows, unsigned cols, unsigned nnz, const unsigned *ptr, const unsigned *col,
                     const double *val, const double *x, double *y, int accumulate) {
    if (!rows) return HBICG_OK;
    if (!g_host_ctx) {
        int rc = hbicg_context_create(&g_host_ctx);
        if (rc) return rc;
    }
    hbicg_matrix *A = NULL;
    int rc = hbicg_matrix_create(g_host_ctx, rows, nnz, ptr, col, val, HBICG_HOST, &A);
    if (rc) return rc;
    cudaStream_t st = g_host_ctx->stream;
    double *dx = NULL, *dy = NULL;
    CUDA_TRY(cudaMalloc((void **)&dx, sizeof(double) * ((size_t)cols + 1)));
    CUDA_TRY(cudaMalloc((void **)&dy, sizeof(double) * ((size_t)rows + 1)));
    if (cols) CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * cols, cudaMemcpyHostToDevice, st));
    if (accumulate) {
        CUDA_TRY(cudaMemcpyAsync(dy, y, sizeof(double) * rows, cudaMemcpyHostToDevice, st));
        HBK_TRY(hbk_spmv_accumulate(&A->k, dx, dy, st));
    } else {
        HBK_TRY(hbk_spmv(&A->k, dx, dy, 0.0, 0, st));
    }
    CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * rows, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(dx);
    cudaFree(dy);
    hbicg_matrix_destroy(A);
    return HBICG_OK;
}

/* ------------------------------------------------------------------------ */
struct hbicg_solver {
    hbicg_context *ctx;
    hbicg_matrix *A;
    int m, kcap, mode;
    hbicg_params p;
    size_t ld;
    hbk_vectors v;
    hbk_shifts sh;
    hbk_scalars *d_sc;
    double *d_sigma, *d_b, *d_res;
    /* plain form */
    double *d_rold, *d_qcopy, *d_r, *d_dot;
    /* fused form graphs */
    cudaGraphExec_t graph;
    int chunk;
    void *tc_ws;      /* tensor-core flush workspace (deferred mode) */
    int *d_tc_err;    /* set by the tensor-core flush on a bounded-wait timeout */
    int launches_per_iter;
    double flush_bytes; /* compulsory HBM bytes of this solve's basis flushes */
    /* deferred mode, pinned host x: solutions that became final at a flush
     * are copied out while the solve goes on */
    double *early_x;        /* the caller's x (host, pinned), or NULL */
    unsigned char *early;   /* [m] row copied */
    int early_pending;      /* copies issued on the context's copy stream */
};

/* After a flush that covered iterations up to k_flushed: shifts that
 * converged by then have their final x_j in the panel-major array (later
 * flushes leave them alone), so each new one is written row-major into X and
 * copied to the caller's buffer on the copy stream, overlapping the rest of
 * the solve. */
static int early_copies(hbicg_solver *s, int k_flushed, int *launches) {
    cudaStream_t st = s->ctx->stream;
    const int m = s->m;
    const unsigned n = s->A->k.n;
    int rc = HBICG_OK, any = 0;
    int *conv = malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!conv) return HBICG_E_NOMEM;
    CUDA_GOTO(cudaMemcpyAsync(conv, s->sh.conv_k, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
    for (int j = 0; j < m; ++j) {
        s->early[j] = s->early[j] ? 1 : 0;
        if (!s->early[j] && conv[j] > 0 && conv[j] <= k_flushed) {
            HBK_GOTO(hbk_panel_row(s->v.Xp, s->v.pm, n, j, s->v.X + (size_t)j * s->ld, st));
            ++*launches;
            s->early[j] = 2; /* written this time: copy below */
            any = 1;
        }
    }
out:
    free(conv);
    if (rc || !any) return rc;
    CUDA_TRY(cudaEventRecord(s->ctx->cev, st));
    CUDA_TRY(cudaStreamWaitEvent(s->ctx->cstream, s->ctx->cev, 0));
    for (int j = 0; j < m; ++j)
        if (s->early[j] == 2) {
            CUDA_TRY(cudaMemcpyAsync(s->early_x + (size_t)j * n, s->v.X + (size_t)j * s->ld, sizeof(double) * n,
                                     cudaMemcpyDeviceToHost, s->ctx->cstream));
            s->early[j] = 1;
        }
    s->early_pending = 1;
    return HBICG_OK;
}

static int pick_mode(const hbicg_params *p, unsigned n, int m) {
    if (p->form == HBICG_FORM_PLAIN) return HBICG_SHIFTS_INCREMENTAL;
    if (p->shift_mode != HBICG_SHIFTS_AUTO) return p->shift_mode;
    /* Deferred mode pays a fixed per-iteration cost (two small kernels and the
     * coefficient update) and saves 4 of 6 FP64 operations per element and
     * shift; it wins once the per-shift vector work dominates. */
    if (m >= 2 && (double)n * (double)m >= (double)(1u << 21)) return HBICG_SHIFTS_DEFERRED;
    return HBICG_SHIFTS_INCREMENTAL;
}

/* Solver buffers come from a library-owned stream-ordered pool per device that
 * keeps freed memory for the next solver (release threshold: unlimited): a
 * one-shot call such as the reference's entry points, which sets up and tears
 * down ~25 GB at 256^3, then neither maps nor unmaps it every time.
 * hbicg_release() returns the cached memory to the device. */
#define HBICG_MAX_DEVICES 64
static cudaMemPool_t g_pools[HBICG_MAX_DEVICES];
static pthread_mutex_t g_pool_lock = PTHREAD_MUTEX_INITIALIZER;

static cudaError_t solver_pool(cudaMemPool_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (dev < 0 || dev >= HBICG_MAX_DEVICES) return cudaErrorInvalidDevice;
    pthread_mutex_lock(&g_pool_lock);
    if (!g_pools[dev]) {
        struct cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        e = cudaMemPoolCreate(&pool, &props);
        if (!e) {
            unsigned long long keep = ~0ull;
            e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            if (!e) g_pools[dev] = pool;
            else cudaMemPoolDestroy(pool);
        }
    }
    *out = g_pools[dev];
    pthread_mutex_unlock(&g_pool_lock);
    return e;
}

/* usable from any stream on return (the allocation's stream is synchronised) */
static cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t st) {
    cudaMemPool_t pool;
    cudaError_t e = solver_pool(&pool);
    if (!e) e = cudaMallocFromPoolAsync(p, bytes > 0 ? bytes : 8, pool, st);
    if (!e) e = cudaStreamSynchronize(st);
    return e;
}

void hbicg_release(void) {
    pthread_mutex_lock(&g_pool_lock);
    for (int d = 0; d < HBICG_MAX_DEVICES; ++d)
        if (g_pools[d]) cudaMemPoolTrimTo(g_pools[d], 0);
    pthread_mutex_unlock(&g_pool_lock);
}

#define DALLOC(ptr, bytes) CUDA_TRY(pool_alloc((void **)&(ptr), (size_t)(bytes), ctx->stream))

int hbicg_solver_create(hbicg_context *ctx, hbicg_matrix *A, int m, const hbicg_params *pp, hbicg_solver **out) {
    hbicg_params p;
    if (pp) p = *pp;
    else hbicg_params_default(&p);
    if (m < 0 || p.max_iter < 0) {
        set_msg("m = %d, max_iter = %d", m, p.max_iter);
        return HBICG_E_ARG;
    }
    hbicg_solver *s = calloc(1, sizeof *s);
    if (!s) return HBICG_E_NOMEM;
    s->ctx = ctx;
    s->A = A;
    s->m = m;
    s->p = p;
    s->kcap = p.max_iter + 1;
    const unsigned n = A->k.n;
    const size_t ld = ld_of(n);
    s->ld = ld;
    const int mm = m > 0 ? m : 1;
    s->mode = pick_mode(&p, n, m);
    size_t vb = sizeof(double) * ld;

    hbk_vectors *v = &s->v;
    memset(v, 0, sizeof *v);
    v->n = n;
    DALLOC(v->r_hat, vb);
    DALLOC(v->s, vb);
    DALLOC(v->y, vb);
    DALLOC(v->X, vb * mm);
    if (s->mode == HBICG_SHIFTS_INCREMENTAL) {
        DALLOC(v->rbuf[0], vb);
        DALLOC(v->rbuf[1], vb);
        DALLOC(v->q, vb);
        DALLOC(v->P, vb * mm);
    } else {
        v->deferred = 1;
        DALLOC(v->ps, vb);
        v->pm = mm;
        DALLOC(v->Xp, sizeof(double) * hbk_panel_elems(n, mm));
        size_t fr = 0, tot = 0;
        CUDA_TRY(cudaMemGetInfo(&fr, &tot));
        double frac = p.basis_mem_frac > 0 ? p.basis_mem_frac : 0.6;
        /* keep room for the flushed p_j (allocated on the first flush) */
        double budget = frac * (double)fr - (double)sizeof(double) * (double)hbk_panel_elems(n, mm);
        long cap = (long)(budget / (double)vb);
        long want = 2L * s->kcap + 8;
        if (cap > want) cap = want;
        /* Blocks of at most 24 iterations by default: the coefficient
         * representation over a long raw Krylov basis loses accuracy where a
         * shift's recurrence nearly breaks down (|pi_k| << |pi_{k-1}|); forming
         * x_j and p_j every block keeps the true residuals at the level of the
         * incremental form (checked on the 256^3 family up to blocks of 32).
         * basis_block < 0 lets the basis grow as far as memory allows. */
        const int block = p.basis_block == 0 ? 24 : p.basis_block;
        if (block > 0 && cap > 2L * block + 3) cap = 2L * block + 3;
        if (cap < 8) {
            /* not enough memory for a useful basis: fall back */
            s->mode = HBICG_SHIFTS_INCREMENTAL;
            v->deferred = 0;
            cudaFreeAsync(v->ps, ctx->stream);
            v->ps = NULL;
            cudaFreeAsync(v->Xp, ctx->stream);
            v->Xp = NULL;
            DALLOC(v->rbuf[0], vb);
            DALLOC(v->rbuf[1], vb);
            DALLOC(v->q, vb);
            DALLOC(v->P, vb * mm);
        } else {
            v->slot_cap = (int)cap;
            DALLOC(v->V, vb * (size_t)cap);
            DALLOC(v->Xc, sizeof(double) * (size_t)mm * (size_t)cap);
            DALLOC(v->Pc, sizeof(double) * (size_t)mm * (size_t)cap);
            DALLOC(v->own, sizeof(double) * 2 * (size_t)mm);
            DALLOC(v->slot_max, sizeof(unsigned long long) * (size_t)cap * HBK_SLOT_SPREAD);
            /* SELL-32 matrices with a stored diagonal in every row: the seed's
             * shift goes onto the diagonal of a private copy of the values,
             * which saves the sigma p and sigma q terms of the two products */
            if (p.form == HBICG_FORM_FUSED && A->k.fmt == HBK_FMT_SELL && A->d_sval && A->k.sell_len) {
                const int drc = sell_diag(A);
                if (drc) return drc;
                if (A->diag_state == 1) {
                    DALLOC(v->sval_shift, sizeof(double) * (size_t)A->k.sell_len);
                    v->sval_orig = A->d_sval;
                    v->sdiag = A->d_sdiag;
                }
            }
            if (p.flush_mode != HBICG_FLUSH_FP64) {
                DALLOC(s->tc_ws, hbk_flush_tc_workspace_bytes(mm));
                DALLOC(s->d_tc_err, sizeof(int));
                CUDA_TRY(cudaMemset(s->d_tc_err, 0, sizeof(int)));
            }
        }
    }

    hbk_shifts *sh = &s->sh;
    memset(sh, 0, sizeof *sh);
    sh->m = m;
    sh->kcap = s->kcap;
    DALLOC(s->d_sc, sizeof(hbk_scalars));
    CUDA_TRY(cudaMemset(s->d_sc, 0, sizeof(hbk_scalars)));
    sh->sc = s->d_sc;
    DALLOC(s->d_sigma, sizeof(double) * mm);
    sh->sigma = s->d_sigma;
    DALLOC(sh->a_hist, sizeof(double) * ((size_t)s->kcap + 1));
    DALLOC(sh->b_hist, sizeof(double) * ((size_t)s->kcap + 1));
    DALLOC(sh->w_hist, sizeof(double) * ((size_t)s->kcap + 1));
    DALLOC(sh->ratio, sizeof(double) * ((size_t)s->kcap + 1));
    DALLOC(sh->rr_hist, sizeof(double) * ((size_t)s->kcap + 1));
    DALLOC(sh->pi, sizeof(double) * (size_t)mm * ((size_t)s->kcap + 1));
    DALLOC(sh->eta, sizeof(double) * mm);
    DALLOC(sh->zeta, sizeof(double) * mm);
    DALLOC(sh->done, sizeof(int) * mm);
    DALLOC(sh->conv_k, sizeof(int) * mm);
    DALLOC(sh->act_list, sizeof(int) * mm);
    DALLOC(sh->lslot, sizeof(int) * mm);
    DALLOC(sh->coef, sizeof(double) * HBK_NCOEF * (size_t)mm);
    DALLOC(sh->sw_k, sizeof(int) * mm);
    DALLOC(sh->sw_seed, sizeof(int) * mm);
    DALLOC(sh->act_hist, sizeof(int) * ((size_t)s->kcap + 1));
    CUDA_TRY(cudaMemset(sh->act_hist, 0, sizeof(int) * ((size_t)s->kcap + 1)));
    size_t nparts = (size_t)(mm > 4 ? mm : 4) * HBK_MAX_GRID;
    DALLOC(sh->partials, sizeof(double) * nparts);
    DALLOC(sh->counters, sizeof(unsigned) * (16 + (size_t)mm));
    CUDA_TRY(cudaMemset(sh->counters, 0, sizeof(unsigned) * (16 + (size_t)mm)));
    DALLOC(s->d_b, vb);
    DALLOC(s->d_res, sizeof(double) * mm);
    DALLOC(s->d_dot, sizeof(double) * 8);
    if (p.form == HBICG_FORM_PLAIN) {
        DALLOC(s->d_rold, vb);
        DALLOC(s->d_qcopy, vb);
        s->d_r = v->rbuf[0];
    }
    s->chunk = p.graph_chunk > 0 ? p.graph_chunk : (n >= (1u << 22) ? 2 : (n >= (1u << 18) ? 4 : 16));
    s->launches_per_iter = s->mode == HBICG_SHIFTS_DEFERRED ? 7 : 5;
    ctx_retain(ctx);
    *out = s;
    return HBICG_OK;
}

void hbicg_solver_destroy(hbicg_solver *s) {
    if (!s) return;
    cudaStreamSynchronize(s->ctx->stream);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    hbk_vectors *v = &s->v;
    hbk_shifts *sh = &s->sh;
    void *ptrs[] = {v->r_hat, v->rbuf[0], v->rbuf[1], v->s, v->q, v->y, v->X, v->P, v->V, v->ps, v->Xc, v->Pc,
                    v->own, v->Pmat, v->Xp, v->slot_max, v->sval_shift, s->d_sc, s->d_sigma, sh->a_hist, sh->b_hist, sh->w_hist, sh->ratio, sh->pi,
                    sh->eta, sh->zeta, sh->done, sh->conv_k, sh->act_list, sh->lslot, sh->coef, sh->sw_k,
                    sh->rr_hist, sh->sw_seed, sh->act_hist, sh->partials, sh->counters, s->d_b, s->d_res, s->d_dot, s->d_rold,
                    s->d_qcopy, s->tc_ws, s->d_tc_err};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++)
        if (ptrs[i]) cudaFreeAsync(ptrs[i], s->ctx->stream); /* back to the pool, in stream order */
    hbicg_context *ctx = s->ctx;
    free(s->early);
    free(s);
    ctx_release(ctx);
}

/* ------------------------------------------------------------------------ */
/* plain form: the reference's iteration, one kernel per step, host scalars */

static int dev_dot(hbicg_solver *s, const double *x, const double *y, double *out) {
    cudaStream_t st = s->ctx->stream;
    HBK_TRY(hbk_dot(s->A->k.n, x, y, s->sh.partials, s->sh.counters + 7, s->d_dot, st));
    CUDA_TRY(cudaMemcpyAsync(s->ctx->h_dbl, s->d_dot, sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *out = s->ctx->h_dbl[0];
    return HBICG_OK;
}

typedef struct {
    int k, n_sw, final_seed, launches, status;
    int *sw_k, *sw_seed, *conv_k, *act;
} plain_out;

static int run_plain(hbicg_solver *s, const double *h_sigma, int seed, plain_out *o) {
    cudaStream_t st = s->ctx->stream;
    const hbk_matrix *A = &s->A->k;
    const unsigned n = A->n;
    const int m = s->m, kcap = s->kcap;
    const size_t ld = s->ld;
    const double tol = s->p.tol;
    hbk_vectors *v = &s->v;
    double *r = s->d_r, *r_old = s->d_rold, *r_hat = v->r_hat, *sv = v->s, *y = v->y, *qc = s->d_qcopy;
    double *ah = malloc(sizeof(double) * (kcap + 1)), *bh = malloc(sizeof(double) * (kcap + 1));
    double *wh = malloc(sizeof(double) * (kcap + 1));
    double *pi = malloc(sizeof(double) * (size_t)m * (kcap + 1));
    double *eta = calloc(m, sizeof(double)), *zeta = malloc(sizeof(double) * m);
    char *done = calloc(m, 1);
    int launches = 0, rc = HBICG_OK;
#define PL(call)                                                                                         \
    do {                                                                                                 \
        launches++;                                                                                      \
        int e_ = (call);                                                                                 \
        if (e_) {                                                                                        \
            set_msg("%s: %s", #call, hbk_error_string(e_));                                              \
            rc = HBICG_E_CUDA;                                                                           \
            goto out;                                                                                    \
        }                                                                                                \
    } while (0)
#define PD(x, y, res)                                                                                    \
    do {                                                                                                 \
        launches++;                                                                                      \
        if ((rc = dev_dot(s, x, y, res))) goto out;                                                      \
    } while (0)

    double rr_hat, rr, bb, rs, qq, qy, rr_hat_old;
    PL(hbk_copy(n, s->d_b, r, st));
    PD(r, r, &rr_hat);
    PL(hbk_copy(n, r, r_hat, st));
    for (int j = 0; j < m; j++) {
        PL(hbk_copy(n, r, v->P + (size_t)j * ld, st));
        zeta[j] = 1.0;
        pi[(size_t)j * kcap + 0] = 1.0;
        if (kcap > 1) pi[(size_t)j * kcap + 1] = 1.0;
    }
    if (cudaMemsetAsync(v->X, 0, sizeof(double) * ld * (size_t)(m > 0 ? m : 1), st) != cudaSuccess) {
        rc = HBICG_E_CUDA;
        goto out;
    }
    rr = bb = rr_hat;
    ah[0] = 1.0;
    bh[0] = 0.0;
    int k = 1, n_done = 0, argmax = seed;
    if (bb == 0.0) n_done = m; /* x = 0 is exact */
    while (n_done < m && k < kcap) {
        double *ps = v->P + (size_t)seed * ld, *xs = v->X + (size_t)seed * ld;
        const double sig_s = h_sigma[seed];
        PL(hbk_copy(n, r, r_old, st));
        PL(hbk_zero(n, sv, st));
        PL(hbk_spmv_accumulate(A, ps, sv, st));
        PL(hbk_axpy(n, sig_s, ps, sv, st));
        PD(r_hat, sv, &rs);
        ah[k] = rr_hat / rs;
        const double ak = ah[k];
        PL(hbk_axpy(n, -ak, sv, r, st));
        PL(hbk_copy(n, r, qc, st));
        PL(hbk_zero(n, y, st));
        PL(hbk_spmv_accumulate(A, r, y, st));
        PL(hbk_axpy(n, sig_s, r, y, st));
        PD(r, r, &qq);
        PD(r, y, &qy);
        wh[k] = qq / qy;
        rr_hat_old = rr_hat;
        const double wk = wh[k];
        PL(hbk_axpy(n, ak, ps, xs, st));
        PL(hbk_axpy(n, wk, r, xs, st));
        PL(hbk_axpy(n, -wk, y, r, st));
        PD(r, r, &rr);
        PD(r_hat, r, &rr_hat);
        bh[k] = (ah[k] / wh[k]) * (rr_hat / rr_hat_old);
        const double bk = bh[k];
        if (!isfinite(ak) || !isfinite(wk) || !isfinite(bk) || wk == 0.0) {
            rc = HBICG_E_BREAKDOWN;
            o->status = HBICG_E_BREAKDOWN;
            break;
        }
        PL(hbk_scal(n, bk, ps, st));
        PL(hbk_axpy(n, 1.0, r, ps, st));
        PL(hbk_axpy(n, -bk * wk, sv, ps, st));
        const double c_prev = (bh[k - 1] / ah[k - 1]) * ak;
        int active = 0;
        for (int j = 0; j < m; j++) {
            if (j == seed || done[j]) continue;
            active++;
            double *pij = pi + (size_t)j * kcap;
            double *xj = v->X + (size_t)j * ld, *pj = v->P + (size_t)j * ld;
            const double d = sig_s - h_sigma[j];
            eta[j] = c_prev * eta[j] - d * ak * pij[k - 1];
            pij[k] = eta[j] + pij[k - 1];
            const double aj = (pij[k - 1] / pij[k]) * ak;
            const double wj = wk / (1.0 - wk * d);
            PL(hbk_axpy(n, wj / (pij[k] * zeta[j]), qc, xj, st));
            PL(hbk_axpy(n, aj, pj, xj, st));
            PL(hbk_axpy(n, wj / (aj * zeta[j] * pij[k]), qc, pj, st));
            PL(hbk_axpy(n, -wj / (aj * zeta[j] * pij[k - 1]), r_old, pj, st));
            zeta[j] = (1.0 - wk * d) * zeta[j];
            const double bj = (pij[k - 1] / pij[k]) * (pij[k - 1] / pij[k]) * bk;
            PL(hbk_scal(n, bj, pj, st));
            PL(hbk_axpy(n, 1.0 / (pij[k] * zeta[j]), r, pj, st));
        }
        if (o->act && k < kcap) o->act[k] = active;
        double best = 1.0;
        for (int j = 0; j < m; j++) {
            if (done[j]) continue;
            const double a = (j == seed) ? 1.0 : fabs(1.0 / (zeta[j] * pi[(size_t)j * kcap + k]));
            if (a * a * rr <= tol * tol * bb) {
                done[j] = 1;
                n_done++;
                if (o->conv_k) o->conv_k[j] = k;
            } else if (a > best) {
                best = a;
                argmax = j;
            }
        }
        if (s->p.switching && done[seed] && n_done < m) {
            const int t = argmax;
            const double *pit = pi + (size_t)t * kcap;
            const double dst = h_sigma[seed] - h_sigma[t];
            for (int i = 1; i <= k; i++) {
                ah[i] = (pit[i - 1] / pit[i]) * ah[i];
                bh[i] = (pit[i - 1] / pit[i]) * (pit[i - 1] / pit[i]) * bh[i];
                wh[i] = wh[i] / (1.0 - wh[i] * dst);
            }
            PL(hbk_scal(n, 1.0 / (zeta[t] * pit[k]), r, st));
            PD(r_hat, r, &rr_hat);
            for (int j = 0; j < m; j++) {
                eta[j] = 0.0;
                zeta[j] = 1.0;
            }
            for (int i = 1; i <= k; i++) {
                for (int j = 0; j < m; j++) {
                    if (done[j] || j == t) continue;
                    double *pij = pi + (size_t)j * kcap;
                    const double d = h_sigma[t] - h_sigma[j];
                    eta[j] = (bh[i - 1] / ah[i - 1]) * ah[i] * eta[j] - d * ah[i] * pij[i - 1];
                    pij[i] = eta[j] + pij[i - 1];
                    zeta[j] = (1.0 - wh[i] * d) * zeta[j];
                }
            }
            seed = t;
            if (o->n_sw < m) {
                if (o->sw_k) o->sw_k[o->n_sw] = k;
                if (o->sw_seed) o->sw_seed[o->n_sw] = t;
            }
            o->n_sw++;
        }
        k++;
    }
    o->k = k;
    o->final_seed = seed;
out:
    o->launches = launches;
    free(ah); free(bh); free(wh); free(pi); free(eta); free(zeta); free(done);
    return rc;
#undef PL
#undef PD
}

/* ------------------------------------------------------------------------ */
/* fused form */

static int capture_graph(hbicg_solver *s) {
    cudaStream_t st = s->ctx->stream;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < s->chunk; i++) {
        int e = hbk_fused_iteration(&s->A->k, &s->v, &s->sh, st);
        if (e) {
            cudaStreamEndCapture(st, &g);
            set_msg("capture: %s", hbk_error_string(e));
            return HBICG_E_CUDA;
        }
    }
    CUDA_TRY(cudaStreamEndCapture(st, &g));
    CUDA_TRY(cudaGraphInstantiate(&s->graph, g, 0));
    cudaGraphDestroy(g);
    return HBICG_OK;
}

static int ensure_pmat(hbicg_solver *s) {
    if (s->v.Pmat) return HBICG_OK;
    const int mm = s->m > 0 ? s->m : 1;
    const size_t bytes = sizeof(double) * hbk_panel_elems(s->A->k.n, mm); /* panel-major */
    CUDA_TRY(pool_alloc((void **)&s->v.Pmat, bytes, s->ctx->stream));
    CUDA_TRY(cudaMemsetAsync(s->v.Pmat, 0, bytes, s->ctx->stream));
    /* the graphs captured the old (null) Pmat pointer: capture again */
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = NULL;
    }
    return HBICG_OK;
}

/* Form x_j (and p_j) from the L basis slots in use: on the tensor cores when
 * the basis fits one K = 64 operand, else with the FP64 kernel; then reset. */
/* k_last: the last iteration the previous flush covered (0 before the first).
 * A shift that converged at or before it has had zero coefficients since
 * that flush, so the tensor-core flush leaves its rows out. */
static int do_flush(hbicg_solver *s, int keep_p, int L, int k_last, int *launches) {
    cudaStream_t st = s->ctx->stream;
    /* basis slots read once; x_j read and written; Pmat_j read (and written),
     * for the shifts the flush forms */
    const double per_shift = keep_p ? 4.0 : 3.0;
    if (s->tc_ws && L >= 1 && L <= hbk_flush_tc_max_slots()) {
        HBK_TRY(hbk_flush_tc_run_live(s->v.V, s->ld, s->A->k.n, L, s->v.Xc, s->v.Pc, s->v.slot_cap, s->v.own, s->m,
                                      s->v.Xp, s->v.Pmat, keep_p, s->sh.conv_k, k_last, s->v.slot_max, s->tc_ws,
                                      s->d_tc_err, st));
        int n_live = 0; /* pageable destination: the copy waits for the flush */
        CUDA_TRY(cudaMemcpyAsync(&n_live, hbk_flush_tc_live_count(s->tc_ws, s->m), sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        s->flush_bytes += 8.0 * s->A->k.n * ((double)L + per_shift * n_live);
        HBK_TRY(hbk_deferred_reset(&s->v, &s->sh, keep_p, st));
        *launches += 5; /* live list, slot maxima, coefficient digits, flush, reset */
    } else {
        s->flush_bytes += 8.0 * s->A->k.n * ((double)L + per_shift * s->m);
        HBK_TRY(hbk_deferred_flush(&s->v, &s->sh, keep_p, st));
        *launches += keep_p ? 3 : 2;
    }
    return HBICG_OK;
}

static int run_fused(hbicg_solver *s, int seed, int *launches, int *flushes, double *flush_ms) {
    cudaStream_t st = s->ctx->stream;
    hbk_scalars *h = s->ctx->h_sc;
    HBK_TRY(hbk_fused_init(&s->A->k, &s->v, &s->sh, s->d_b, seed, s->p.tol, st));
    /* switching flag lives in the device scalars */
    int sw = s->p.switching ? 1 : 0;
    CUDA_TRY(cudaMemcpyAsync(&s->d_sc->switching, &sw, sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *launches += 6 + (s->v.deferred ? 1 : s->m);
    const int use_graph = s->p.use_graph;
    /* every launch of a chunk advances k by chunk unless the solve ends or
     * the basis pauses it; bound the host loop all the same */
    long guard = 0;
    const long guard_max = 4L * s->kcap / s->chunk + 64;
    int k_flushed = 0; /* last iteration covered by a flush */
    for (;;) {
        if (++guard > guard_max) {
            set_msg("fused loop made no progress after %ld chunks", guard_max);
            return HBICG_E_TIMEOUT;
        }
        if (use_graph) {
            if (!s->graph) {
                int rc = capture_graph(s);
                if (rc) return rc;
            }
            CUDA_TRY(cudaGraphLaunch(s->graph, st));
        } else {
            for (int i = 0; i < s->chunk; i++) HBK_TRY(hbk_fused_iteration(&s->A->k, &s->v, &s->sh, st));
        }
        *launches += s->chunk * s->launches_per_iter;
        CUDA_TRY(cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (!h->finished) continue;
        if ((h->status & HBK_ST_BASIS_FULL) && !(h->status & HBK_ST_BREAKDOWN)) {
            int rc = ensure_pmat(s);
            if (rc) return rc;
            float t = 0.f;
            CUDA_TRY(cudaEventRecord(s->ctx->evf0, st));
            rc = do_flush(s, 1, h->slots, k_flushed, launches);
            if (rc) return rc;
            k_flushed = h->k - 1;
            if (s->early_x && (rc = early_copies(s, k_flushed, launches))) return rc;
            CUDA_TRY(cudaEventRecord(s->ctx->evf1, st));
            CUDA_TRY(cudaEventSynchronize(s->ctx->evf1));
            CUDA_TRY(cudaEventElapsedTime(&t, s->ctx->evf0, s->ctx->evf1));
            *flush_ms += t;
            (*flushes)++;
            continue;
        }
        break;
    }
    if (s->v.deferred) {
        float t = 0.f;
        CUDA_TRY(cudaEventRecord(s->ctx->evf0, st));
        int rc = do_flush(s, 0, h->slots, k_flushed, launches);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(s->ctx->evf1, st));
        /* x_j were panel-major during the solve; rows already on their way to
         * the host are rewritten with the same values only after those copies */
        if (s->early_pending) {
            CUDA_TRY(cudaEventRecord(s->ctx->cev, s->ctx->cstream));
            CUDA_TRY(cudaStreamWaitEvent(st, s->ctx->cev, 0));
        }
        HBK_TRY(hbk_panel_to_rows(s->v.Xp, s->v.pm, s->A->k.n, s->v.X, s->ld, st));
        ++*launches;
        CUDA_TRY(cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, st));
        int tc_err = 0;
        if (s->d_tc_err) CUDA_TRY(cudaMemcpyAsync(&tc_err, s->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaEventElapsedTime(&t, s->ctx->evf0, s->ctx->evf1));
        *flush_ms += t;
        if (tc_err) {
            set_msg("tensor-core flush: an mbarrier wait timed out");
            return HBICG_E_TIMEOUT;
        }
        return HBICG_OK;
    }
    CUDA_TRY(cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return HBICG_OK;
}

/* compulsory HBM bytes of the fused schedule for one solve */
static double algorithmic_bytes(const hbicg_solver *s, int k_end, const int *act) {
    const double n = s->A->k.n, nnz = s->A->k.nnz;
    const double spmv = 12.0 * nnz + 4.0 * (n + 1) + 16.0 * n;
    double tot = 0.0;
    for (int k = 1; k < k_end; k++) {
        const double ma = act ? act[k] : 0;
        if (s->mode == HBICG_SHIFTS_DEFERRED) tot += 2.0 * spmv + 8.0 * n * 13.0;
        else tot += 2.0 * spmv + 8.0 * n * 17.0 + 32.0 * n * ma;
    }
    if (s->mode == HBICG_SHIFTS_DEFERRED) tot += 8.0 * n * (2.0 * (k_end - 1) + 1.0) + 8.0 * n * s->m;
    return tot;
}

/* Host output memory that was never written (fresh malloc / numpy.zeros
 * pages) is faulted in page by page inside CUDA's pageable device-to-host
 * copy, which on the GB300 host costs ~1 ms per MB (55 ms for 59 MB, more
 * than the solve of that family).  Touching one byte per page from a helper
 * thread while the GPU solves takes the normal page-fault path instead. */
typedef struct {
    char *p[2];
    size_t bytes[2];
    pthread_t th;
    int active;
} touch_t;

static void touch_join(touch_t *t) {
    if (t->active) {
        pthread_join(t->th, NULL);
        t->active = 0;
    }
}

static void *touch_pages(void *arg) {
    const touch_t *t = arg;
    long pg = sysconf(_SC_PAGESIZE);
    if (pg <= 0) pg = 4096;
    for (int i = 0; i < 2; i++) {
        volatile char *p = t->p[i];
        if (!p || !t->bytes[i]) continue;
        for (size_t o = 0; o < t->bytes[i]; o += (size_t)pg) p[o] = 0;
        p[t->bytes[i] - 1] = 0;
    }
    return NULL;
}

/* host scratch of one solve, freed by the caller on every return path */
typedef struct {
    double *h_sigma, *h_res;
    int *act, *sw_k, *sw_seed, *conv;
    unsigned char *fixed;
} run_host_t;

static void run_host_free(run_host_t *hb) {
    free(hb->h_sigma);
    free(hb->h_res);
    free(hb->act);
    free(hb->sw_k);
    free(hb->sw_seed);
    free(hb->conv);
    free(hb->fixed);
    memset(hb, 0, sizeof *hb);
}

static int solver_run_impl(hbicg_solver *s, const double *b, const double *sigma, int seed, int in_where, double *x,
                           double *r_out, int out_where, hbicg_stats *stats, touch_t *touch, run_host_t *hb);

/* params.refine: true residuals of every shift; a shift above tol gets
 * x_j += e with (A + sigma_j I) e = b - (A + sigma_j I) x_j solved (single
 * shift, incremental form) to 0.5 tol ||b|| / ||r_j||; at most 3 rounds. */
static int refine_shifts(hbicg_solver *s, const double *h_sigma, int *refined, unsigned char *fixed) {
    cudaStream_t st = s->ctx->stream;
    const unsigned n = s->A->k.n;
    const int m = s->m;
    const size_t ld = s->ld;
    double *h = malloc(sizeof(double) * (size_t)m), *r = NULL, *e = NULL;
    hbicg_solver *sub = NULL;
    int rc = HBICG_OK;
    if (!h) return HBICG_E_NOMEM;
    HBK_GOTO(hbk_dot(n, s->d_b, s->d_b, s->sh.partials, s->sh.counters + 7, s->d_dot, st));
    CUDA_GOTO(cudaMemcpyAsync(s->ctx->h_dbl, s->d_dot, sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_GOTO(cudaStreamSynchronize(st));
    const double bn = sqrt(s->ctx->h_dbl[0]);
    for (int round = 0; round < 3 && rc == HBICG_OK && bn > 0.0; ++round) {
        HBK_GOTO(hbk_true_residuals(&s->A->k, s->v.X, s->d_b, s->d_sigma, m, s->sh.partials, s->sh.counters + 16,
                                   s->d_res, st));
        CUDA_GOTO(cudaMemcpyAsync(h, s->d_res, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, st));
        CUDA_GOTO(cudaStreamSynchronize(st));
        int any = 0;
        for (int j = 0; j < m && rc == HBICG_OK; ++j) {
            const double res = sqrt(h[j]) / bn;
            if (res <= s->p.tol) continue;
            any = 1;
            if (!r) {
                CUDA_GOTO(cudaMalloc((void **)&r, sizeof(double) * ((size_t)n + 1)));
                CUDA_GOTO(cudaMalloc((void **)&e, sizeof(double) * ((size_t)n + 1)));
            }
            if (!sub) {
                hbicg_params p1 = s->p;
                p1.refine = 0;
                p1.true_residuals = 0;
                p1.shift_mode = HBICG_SHIFTS_INCREMENTAL;
                if ((rc = hbicg_solver_create(s->ctx, s->A, 1, &p1, &sub)) != HBICG_OK) break;
            }
            double *xj = s->v.X + (size_t)j * ld;
            HBK_GOTO(hbk_spmv(&s->A->k, xj, e, h_sigma[j], 1, st)); /* e = (A + sigma_j I) x_j */
            HBK_GOTO(hbk_copy(n, s->d_b, r, st));
            HBK_GOTO(hbk_axpy(n, -1.0, e, r, st));                   /* r = b - e */
            sub->p.tol = isfinite(res) ? 0.5 * s->p.tol / res : s->p.tol;
            const int sr = hbicg_solver_run(sub, r, s->d_sigma + j, 0, HBICG_DEVICE, e, NULL, HBICG_DEVICE, NULL);
            if (sr != HBICG_OK && sr != HBICG_E_MAXITER) {
                rc = sr;
                break;
            }
            HBK_GOTO(hbk_axpy(n, 1.0, e, xj, st));
            ++*refined;
            if (fixed) fixed[j] = 1;
        }
        if (!any) break;
    }
out:
    hbicg_solver_destroy(sub);
    cudaFree(r);
    cudaFree(e);
    free(h);
    return rc;
}

/* the page-touching helper is joined, and the host scratch freed, on every
 * return path of the solve */
int hbicg_solver_run(hbicg_solver *s, const double *b, const double *sigma, int seed, int in_where, double *x,
                     double *r_out, int out_where, hbicg_stats *stats) {
    touch_t touch;
    memset(&touch, 0, sizeof touch);
    run_host_t hb;
    memset(&hb, 0, sizeof hb);
    const int rc = solver_run_impl(s, b, sigma, seed, in_where, x, r_out, out_where, stats, &touch, &hb);
    touch_join(&touch);
    run_host_free(&hb);
    /* no copy into the caller's buffer outlives the call, whatever path returned */
    if (s->early_pending) cudaStreamSynchronize(s->ctx->cstream);
    s->early_x = NULL;
    s->early_pending = 0;
    free(s->early);
    s->early = NULL;
    return rc;
}

static int solver_run_impl(hbicg_solver *s, const double *b, const double *sigma, int seed, int in_where, double *x,
                           double *r_out, int out_where, hbicg_stats *stats, touch_t *touch, run_host_t *hb) {
    hbicg_context *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const unsigned n = s->A->k.n;
    const int m = s->m;
    if (m > 0 && (seed < 0 || seed >= m)) {
        set_msg("seed %d out of range [0, %d)", seed, m);
        return HBICG_E_ARG;
    }
    const enum cudaMemcpyKind kin = in_where == HBICG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const enum cudaMemcpyKind kout = out_where == HBICG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    double *h_sigma = hb->h_sigma = malloc(sizeof(double) * (m > 0 ? m : 1));
    int *act = hb->act = calloc((size_t)s->kcap + 1, sizeof(int));
    int *sw_k = hb->sw_k = calloc(m > 0 ? m : 1, sizeof(int)), *sw_seed = hb->sw_seed = calloc(m > 0 ? m : 1, sizeof(int));
    int *conv = hb->conv = calloc(m > 0 ? m : 1, sizeof(int));
    if (!h_sigma || !act || !sw_k || !sw_seed || !conv) {
        set_msg("host scratch of %d shifts and %d iterations", m, s->kcap);
        return HBICG_E_NOMEM;
    }
    if (m > 0) {
        if (in_where == HBICG_DEVICE) CUDA_TRY(cudaMemcpyAsync(h_sigma, sigma, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        else memcpy(h_sigma, sigma, sizeof(double) * m);
        CUDA_TRY(cudaMemcpyAsync(s->d_sigma, sigma, sizeof(double) * m, kin, st));
    }
    CUDA_TRY(cudaMemcpyAsync(s->d_b, b, sizeof(double) * n, kin, st));
    /* pinned host x needs no page touching; in deferred mode its finished rows
     * are copied out during the solve */
    int x_pinned = 0;
    if (out_where != HBICG_DEVICE && x && m > 0) {
        struct cudaPointerAttributes pa;
        x_pinned = cudaPointerGetAttributes(&pa, x) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        cudaGetLastError(); /* an unregistered pointer is not an error here */
    }
    /* host outputs: fault their pages in while the GPU solves (the inputs are
     * consumed first, in case an output buffer also held an input) */
    if (out_where != HBICG_DEVICE && ((x && m > 0 && !x_pinned) || r_out)) {
        CUDA_TRY(cudaStreamSynchronize(st));
        touch->p[0] = x_pinned ? NULL : (char *)x;
        touch->bytes[0] = x && !x_pinned ? sizeof(double) * (size_t)n * (size_t)(m > 0 ? m : 0) : 0;
        touch->p[1] = (char *)r_out;
        touch->bytes[1] = r_out ? sizeof(double) * (size_t)n : 0;
        if (touch->bytes[0] + touch->bytes[1] >= (1u << 20) && pthread_create(&touch->th, NULL, touch_pages, touch) == 0)
            touch->active = 1;
        else
            touch_pages(touch);
    }
    /* deferred mode into pinned host memory: copy finished solutions out
     * during the solve (pageable copies would block the thread driving it) */
    s->early_x = NULL;
    s->early_pending = 0;
    free(s->early);
    s->early = NULL;
    if (s->p.form != HBICG_FORM_PLAIN && s->v.deferred && x_pinned && (s->early = calloc((size_t)m, 1)) != NULL)
        s->early_x = x;
    CUDA_TRY(cudaEventRecord(ctx->ev0, st));
    int rc = HBICG_OK, launches = 0, flushes = 0;
    double flush_ms = 0.0;
    s->flush_bytes = 0.0;
    int k = 1, n_sw = 0, final_seed = seed, status = HBICG_OK;
    const double *r_final = NULL;
    if (s->p.form == HBICG_FORM_PLAIN) {
        plain_out o;
        memset(&o, 0, sizeof o);
        o.sw_k = sw_k;
        o.sw_seed = sw_seed;
        o.conv_k = conv;
        o.act = act;
        rc = run_plain(s, h_sigma, seed, &o);
        k = o.k;
        n_sw = o.n_sw;
        final_seed = o.final_seed;
        launches = o.launches;
        if (rc == HBICG_E_BREAKDOWN) {
            status = rc;
            rc = HBICG_OK;
        }
        r_final = s->d_r;
    } else {
        rc = run_fused(s, seed, &launches, &flushes, &flush_ms);
        if (rc == HBICG_OK) {
            hbk_scalars *h = ctx->h_sc;
            k = h->k;
            n_sw = h->n_sw;
            final_seed = h->seed;
            if (h->status & HBK_ST_BREAKDOWN) status = HBICG_E_BREAKDOWN;
            if (m > 0) {
                CUDA_TRY(cudaMemcpyAsync(conv, s->sh.conv_k, sizeof(int) * m, cudaMemcpyDeviceToHost, st));
                int nl = n_sw < m ? n_sw : m;
                if (nl) {
                    CUDA_TRY(cudaMemcpyAsync(sw_k, s->sh.sw_k, sizeof(int) * nl, cudaMemcpyDeviceToHost, st));
                    CUDA_TRY(cudaMemcpyAsync(sw_seed, s->sh.sw_seed, sizeof(int) * nl, cudaMemcpyDeviceToHost, st));
                }
            }
            CUDA_TRY(cudaMemcpyAsync(act, s->sh.act_hist, sizeof(int) * ((size_t)s->kcap + 1), cudaMemcpyDeviceToHost, st));
            r_final = s->v.deferred ? s->v.V + (size_t)h->slot_r_old * s->ld : s->v.rbuf[(h->k - 1) & 1];
        }
    }
    CUDA_TRY(cudaEventRecord(ctx->ev1, st));
    /* copies issued during the solve finish before anything rewrites X */
    if (s->early_pending) CUDA_TRY(cudaStreamSynchronize(ctx->cstream));
    int refined = 0;
    unsigned char *fixed = hb->fixed = s->early_x ? calloc((size_t)m, 1) : NULL;
    /* only after a converged solve: a solve stopped by max_iter or a breakdown
     * keeps its x as the reference leaves it */
    if (rc == HBICG_OK && status == HBICG_OK && s->p.refine && m > 0 && k < s->kcap) {
        rc = refine_shifts(s, h_sigma, &refined, fixed);
        CUDA_TRY(cudaEventRecord(ctx->ev1, st)); /* solve_ms includes the corrections */
    }
    touch_join(touch);
    if (rc == HBICG_OK && x && m > 0) {
        if (s->early_x && s->early && fixed) {
            /* the rows not copied during the solve, and the corrected ones */
            for (int j = 0; j < m; ++j)
                if (!s->early[j] || fixed[j])
                    CUDA_TRY(cudaMemcpyAsync(x + (size_t)j * n, s->v.X + (size_t)j * s->ld, sizeof(double) * n,
                                             kout, st));
        } else {
            CUDA_TRY(cudaMemcpy2DAsync(x, sizeof(double) * n, s->v.X, sizeof(double) * s->ld, sizeof(double) * n, m,
                                       kout, st));
        }
    }
    if (rc == HBICG_OK && r_out && r_final) CUDA_TRY(cudaMemcpyAsync(r_out, r_final, sizeof(double) * n, kout, st));
    double maxres = 0.0;
    double *h_res = NULL;
    if (rc == HBICG_OK && s->p.true_residuals && m > 0) {
        HBK_TRY(hbk_true_residuals(&s->A->k, s->v.X, s->d_b, s->d_sigma, m, s->sh.partials, s->sh.counters + 16,
                                   s->d_res, st));
        HBK_TRY(hbk_dot(n, s->d_b, s->d_b, s->sh.partials, s->sh.counters + 7, s->d_dot, st));
        if (!(h_res = hb->h_res = malloc(sizeof(double) * m))) {
            set_msg("host scratch of %d residuals", m);
            return HBICG_E_NOMEM;
        }
        CUDA_TRY(cudaMemcpyAsync(h_res, s->d_res, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(ctx->h_dbl, s->d_dot, sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    if (h_res) {
        const double bn = sqrt(ctx->h_dbl[0]);
        for (int j = 0; j < m; j++) {
            h_res[j] = sqrt(h_res[j]) / bn;
            if (h_res[j] > maxres || isnan(h_res[j])) maxres = h_res[j];
        }
    }
    if (rc == HBICG_OK && status == HBICG_OK && k >= s->kcap && m > 0) {
        int all = 1;
        for (int j = 0; j < m; j++)
            if (!conv[j]) all = 0;
        if (!all) status = HBICG_E_MAXITER;
    }
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->k = k;
        stats->status = rc ? rc : status;
        stats->n_switches = n_sw;
        stats->final_seed = final_seed;
        stats->shift_mode = s->mode;
        stats->basis_flushes = flushes;
        stats->launches = launches;
        stats->refined_shifts = refined;
        stats->solve_ms = ms;
        stats->flush_ms = flush_ms;
        stats->max_true_residual = maxres;
        stats->bytes_algorithmic = algorithmic_bytes(s, k, act);
        stats->flush_bytes = s->flush_bytes;
        int nl = n_sw < m ? n_sw : m;
        if (stats->switch_k) memcpy(stats->switch_k, sw_k, sizeof(int) * nl);
        if (stats->switch_seed) memcpy(stats->switch_seed, sw_seed, sizeof(int) * nl);
        if (stats->conv_k && m > 0) memcpy(stats->conv_k, conv, sizeof(int) * m);
        if (stats->active_per_iter) memcpy(stats->active_per_iter, act, sizeof(int) * ((size_t)s->kcap + 1));
        if (stats->true_residual && h_res) memcpy(stats->true_residual, h_res, sizeof(double) * m);
        if (s->p.form == HBICG_FORM_FUSED && k > 0) {
            const size_t nk = (size_t)(k < s->kcap ? k : s->kcap);
            if (stats->seed_alpha) cudaMemcpy(stats->seed_alpha, s->sh.a_hist, sizeof(double) * nk, cudaMemcpyDeviceToHost);
            if (stats->seed_beta) cudaMemcpy(stats->seed_beta, s->sh.b_hist, sizeof(double) * nk, cudaMemcpyDeviceToHost);
            if (stats->seed_omega) cudaMemcpy(stats->seed_omega, s->sh.w_hist, sizeof(double) * nk, cudaMemcpyDeviceToHost);
            if (stats->seed_rr) cudaMemcpy(stats->seed_rr, s->sh.rr_hist, sizeof(double) * nk, cudaMemcpyDeviceToHost);
        }
    }
    if (rc) return rc;
    return status;
}

int hbicg_solve(unsigned n, unsigned nnz, const unsigned *ptr, const unsigned *col, const double *val,
                const double *b, const double *sigma, int m, int seed, const hbicg_params *p, double *x,
                double *r_out, hbicg_stats *stats) {
    hbicg_context *ctx = NULL;
    hbicg_matrix *A = NULL;
    hbicg_solver *s = NULL;
    int rc = hbicg_context_create(&ctx);
    if (!rc) rc = hbicg_matrix_create(ctx, n, nnz, ptr, col, val, HBICG_HOST, &A);
    if (!rc) rc = hbicg_solver_create(ctx, A, m, p, &s);
    if (!rc) rc = hbicg_solver_run(s, b, sigma, seed, HBICG_HOST, x, r_out, HBICG_HOST, stats);
    hbicg_solver_destroy(s);
    hbicg_matrix_destroy(A);
    hbicg_context_destroy(ctx);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* the reference's entry points (src/solver.h:33-35) */

static double g_tol = EPS;
static int g_maxit = MAX_ITER;
static int g_switching = 1;

void hbicg_dropin_config(double tol, int max_iter, int switching) {
    g_tol = tol;
    g_maxit = max_iter;
    g_switching = switching;
}

/* A_loc_offd holds global column indices (src/matrix.c:387-389); on one rank
 * it is empty.  A non-empty one is merged row by row after the diagonal
 * block's entries. */
static int merged_csr(const CSR_Matrix *d, const CSR_Matrix *o, unsigned **ptr, unsigned **col, double **val) {
    const unsigned n = d->rows;
    const unsigned nz = d->nz + o->nz;
    *ptr = malloc(sizeof(unsigned) * ((size_t)n + 1));
    *col = malloc(sizeof(unsigned) * ((size_t)nz + 1));
    *val = malloc(sizeof(double) * ((size_t)nz + 1));
    if (!*ptr || !*col || !*val) return HBICG_E_NOMEM;
    unsigned e = 0;
    (*ptr)[0] = 0;
    for (unsigned i = 0; i < n; i++) {
        for (unsigned a = d->ptr[i]; a < d->ptr[i + 1]; a++) {
            (*col)[e] = d->col[a];
            (*val)[e++] = d->val[a];
        }
        for (unsigned a = o->ptr[i]; a < o->ptr[i + 1]; a++) {
            (*col)[e] = o->col[a];
            (*val)[e++] = o->val[a];
        }
        (*ptr)[i + 1] = e;
    }
    return HBICG_OK;
}

static int dropin(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                  double *r_loc, double *sigma, int sigma_len, int seed, int form, int use_graph) {
    if (A_info->cols != A_info->rows) {
        printf("Error: matrix is not square.\n");
        exit(1);
    }
    hbicg_params p;
    hbicg_params_default(&p);
    p.tol = g_tol;
    p.max_iter = g_maxit;
    p.switching = g_switching;
    p.form = form;
    p.use_graph = use_graph;
    p.refine = 0; /* the reference's entry points return the reference's x */
    const CSR_Matrix *A = A_loc_diag;
    unsigned *ptr = A->ptr, *col = A->col;
    double *val = A->val;
    int merged = 0;
    if (A_loc_offd && A_loc_offd->nz > 0 && A_loc_offd->ptr) {
        int rc = merged_csr(A_loc_diag, A_loc_offd, &ptr, &col, &val);
        if (rc) return -rc;
        merged = 1;
    }
    hbicg_stats st;
    memset(&st, 0, sizeof st);
    const unsigned nz = ptr[A->rows];
    int rc = hbicg_solve(A->rows, nz, ptr, col, val, r_loc, sigma, sigma_len, seed, &p, x_loc_set, r_loc, &st);
    if (merged) {
        free(ptr);
        free(col);
        free(val);
    }
    if (rc != HBICG_OK && rc != HBICG_E_MAXITER && rc != HBICG_E_BREAKDOWN) {
        fprintf(stderr, "hbicg: %s (%s)\n", hbicg_status_string(rc), hbicg_last_message());
        return -rc;
    }
    return st.k;
}

int shifted_lopbicg_dynamic(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                            double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_FUSED, 1);
}

int shifted_lopbicg_static(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_PLAIN, 0);
}

int shifted_lopbicg_normal(CSR_Matrix *A_loc_diag, CSR_Matrix *A_loc_offd, INFO_Matrix *A_info, double *x_loc_set,
                           double *r_loc, double *sigma, int sigma_len, int seed) {
    return dropin(A_loc_diag, A_loc_offd, A_info, x_loc_set, r_loc, sigma, sigma_len, seed, HBICG_FORM_FUSED, 0);
}
