/* Host driver of the GB300 shifted BiCGStab solver (C11 + CUDA runtime):
 * contexts, the solver's device workspace and its runs.  Matrices and their
 * SpMV forms are in matrix_forms.c, the reference's entry points
 * (src/solver.h:33-35) in dropin.c.
 *
 * A solver owns the device workspace, uploads inputs, runs one of the two
 * iteration forms and returns results through the extended API
 * (include/hbicg.h):
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

#include "host_internal.h"
#include "solver.h"

/* ------------------------------------------------------------------------ */
static _Thread_local char g_msg[512];

void hbicg__set_msg(const char *fmt, ...) {
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

void hbicg__ctx_retain(hbicg_context *c) { __atomic_add_fetch(&c->refs, 1, __ATOMIC_RELAXED); }
static void ctx_free(hbicg_context *c);
/* the context is freed when its handle and every matrix and solver made on it
 * are gone, in whatever order a caller (or a garbage collector) destroys them */
void hbicg__ctx_release(hbicg_context *c) {
    if (__atomic_sub_fetch(&c->refs, 1, __ATOMIC_ACQ_REL) == 0) ctx_free(c);
}

int hbicg_context_create(hbicg_context **out) { return hbicg__context_create_prio(out, 0); }

/* high = 1: the context's stream at the device's greatest priority, so that
 * its short steps are scheduled ahead of other streams' pending blocks */
int hbicg__context_create_prio(hbicg_context **out, int high) {
    hbicg_context *c = calloc(1, sizeof *c);
    if (!c) return HBICG_E_NOMEM;
    c->refs = 1;
    int rc = HBICG_OK, lo = 0, hi = 0;
    if (high && cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess)
        CUDA_GOTO(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, hi));
    else
        CUDA_GOTO(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUDA_GOTO(cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
    CUDA_GOTO(cudaEventCreateWithFlags(&c->cev, cudaEventDisableTiming));
    CUDA_GOTO(cudaEventCreate(&c->ev0));
    CUDA_GOTO(cudaEventCreate(&c->ev1));
    CUDA_GOTO(cudaEventCreate(&c->evf0));
    CUDA_GOTO(cudaEventCreate(&c->evf1));
    CUDA_GOTO(cudaMallocHost((void **)&c->h_sc, sizeof(hbk_scalars)));
    CUDA_GOTO(cudaMallocHost((void **)&c->h_dbl, sizeof(double) * 64));
    *out = c;
    return HBICG_OK;
out: /* release what was made before the failing call */
    if (c->h_sc) cudaFreeHost(c->h_sc);
    if (c->evf1) cudaEventDestroy(c->evf1);
    if (c->evf0) cudaEventDestroy(c->evf0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->cev) cudaEventDestroy(c->cev);
    if (c->cstream) cudaStreamDestroy(c->cstream);
    if (c->stream) cudaStreamDestroy(c->stream);
    free(c);
    return rc;
}

void hbicg_context_destroy(hbicg_context *c) {
    if (c) hbicg__ctx_release(c);
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
    int graph_loop;    /* graph is one conditional while loop over iterations */
    int no_loop_graph; /* the runtime refused the loop graph: chunks of iterations */
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

int hbicg__shift_mode_for(const hbicg_params *p, unsigned n, int m) { return pick_mode(p, n, m); }

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

/* the same pool for the matrices' device arrays (the CSR copy and the SELL-32
 * form): a one-shot call such as the reference's entry points then reuses the
 * memory of the previous call instead of mapping ~3 GB again at 256^3 */
cudaError_t hbicg__dev_alloc(void **p, size_t bytes, cudaStream_t st) { return pool_alloc(p, bytes, st); }

/* back to the pool in stream order (p from hbicg__dev_alloc, or NULL) */
void hbicg__dev_free(void *p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
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
    const size_t ld = hbicg__ld_of(n);
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
        /* Blocks of at most 28 iterations by default (59 slots: within the
         * tensor-core flush's 64): the coefficient representation over a long
         * raw Krylov basis loses accuracy where a shift's recurrence nearly
         * breaks down (|pi_k| << |pi_{k-1}|); forming x_j and p_j every block
         * keeps the true residuals at the level of the incremental form.
         * Measured on the 256^3 family: blocks of 24 and 28 end at the same
         * residuals and solutions (28: 15 flushes instead of 18, 0.776 against
         * 0.827 s); 26 left one shift for the true-residual correction, 30
         * misses the tolerance.  basis_block < 0 lets the basis grow as far as
         * memory allows. */
        const int block = p.basis_block == 0 ? 28 : p.basis_block;
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
                const int drc = hbicg__sell_diag(A);
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
    hbicg__ctx_retain(ctx);
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
    hbicg__ctx_release(ctx);
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
    int k = 1, n_done = 0, argmax = seed, shift_fail = 0;
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
            const double e_new = c_prev * eta[j] - d * ak * pij[k - 1];
            const double pik = e_new + pij[k - 1];
            const double den = 1.0 - wk * d;
            const double aj = (pij[k - 1] / pik) * ak;
            const double wj = wk / den;
            const double zn = den * zeta[j];
            const double c0 = wj / (pik * zeta[j]), c2 = wj / (aj * zeta[j] * pik);
            const double c3 = -wj / (aj * zeta[j] * pij[k - 1]);
            const double bj = (pij[k - 1] / pik) * (pij[k - 1] / pik) * bk, c5 = 1.0 / (pik * zn);
            /* shift breakdown: pi_k = 0, 1 - omega d = 0 or a non-finite
             * scalar; the shift keeps its last finite iterate and stops */
            if (pik == 0.0 || den == 0.0 || !isfinite(e_new) || !isfinite(zn) || !isfinite(c0) || !isfinite(aj) ||
                !isfinite(c2) || !isfinite(c3) || !isfinite(bj) || !isfinite(c5)) {
                done[j] = 1;
                n_done++;
                shift_fail = 1;
                if (o->conv_k) o->conv_k[j] = -k;
                continue;
            }
            eta[j] = e_new;
            pij[k] = pik;
            PL(hbk_axpy(n, c0, qc, xj, st));
            PL(hbk_axpy(n, aj, pj, xj, st));
            PL(hbk_axpy(n, c2, qc, pj, st));
            PL(hbk_axpy(n, c3, r_old, pj, st));
            zeta[j] = zn;
            PL(hbk_scal(n, bj, pj, st));
            PL(hbk_axpy(n, c5, r, pj, st));
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
    if (shift_fail && rc == HBICG_OK) {
        rc = HBICG_E_BREAKDOWN;
        o->status = HBICG_E_BREAKDOWN;
    }
out:
    o->launches = launches;
    free(ah); free(bh); free(wh); free(pi); free(eta); free(zeta); free(done);
    return rc;
#undef PL
#undef PD
}

/* ------------------------------------------------------------------------ */
/* fused form */

/* The iterations as one conditional while node: its body is `chunk`
 * iterations followed by a one-thread kernel that sets the loop's condition
 * to "not finished", so a graph launch runs iterations until the solve
 * converges, reaches max_iter, breaks down or needs a basis flush, with no
 * host round trip in between.  Iterations after the stop inside a body find
 * the solve finished and return at once (as in a chunk graph).  More than one
 * iteration per body because every body costs a device-side graph launch:
 * at one iteration per body, families of 10^4..10^5 rows (iterations of
 * 20..60 us) ran 35 % slower than with chunk graphs and a host check per
 * chunk.  Opt-in (params.use_graph = 2): measured on GB300 it matches chunk
 * graphs on single solves (32^3: 4.81 against 4.83 ms; 256^3: 0.8256 against
 * 0.8268 s) and loses when several families share the GPU (256 families on
 * 8 host workers: 2.36 against 1.98 s).  The loop is also bounded by a count of bodies per solve
 * (2 kcap + 64: every relaunch after a flush adds at most one body that finds
 * the solve stopped).  Returns nonzero, with nothing left behind, when the
 * runtime refuses any step; the caller then captures chunks of iterations. */
static int capture_loop_graph(hbicg_solver *s) {
    cudaStream_t st = s->ctx->stream;
    cudaGraph_t g = NULL, body_out = NULL;
    cudaGraphExec_t ex = NULL;
    cudaGraphConditionalHandle cond;
    cudaGraphNode_t node;
    struct cudaGraphNodeParams np;
    int capturing = 0, ok = 0;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) goto out;
    if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) goto out;
    memset(&np, 0, sizeof np);
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, NULL, NULL, 0, &np) != cudaSuccess) goto out;
    if (cudaStreamBeginCaptureToGraph(st, np.conditional.phGraph_out[0], NULL, NULL, 0,
                                      cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        goto out;
    capturing = 1;
    for (int i = 0; i < s->chunk; i++)
        if (hbk_fused_iteration(&s->A->k, &s->v, &s->sh, st)) goto out;
    if (hbk_loop_condition(&s->sh, cond, 2 * s->kcap + 64, st)) goto out;
    capturing = 0;
    if (cudaStreamEndCapture(st, &body_out) != cudaSuccess) goto out;
    if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) goto out;
    s->graph = ex;
    s->graph_loop = 1;
    ok = 1;
out:
    if (capturing) cudaStreamEndCapture(st, &body_out);
    if (g) cudaGraphDestroy(g);
    if (!ok) cudaGetLastError(); /* a refused step leaves no error behind for later calls */
    return ok ? 0 : 1;
}

static int capture_graph(hbicg_solver *s) {
    cudaStream_t st = s->ctx->stream;
    cudaGraph_t g;
    if (s->p.use_graph == 2 && !s->no_loop_graph && capture_loop_graph(s) == 0) return HBICG_OK;
    s->no_loop_graph = 1; /* refused once: chunks from now on */
    s->graph_loop = 0;
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

/* first step of a fused solve: the device scalars, r and p_j (or the basis) from b */
static int fused_init(hbicg_solver *s, int seed, int *launches) {
    cudaStream_t st = s->ctx->stream;
    HBK_TRY(hbk_fused_init(&s->A->k, &s->v, &s->sh, s->d_b, seed, s->p.tol, st));
    /* switching flag lives in the device scalars */
    int sw = s->p.switching ? 1 : 0;
    CUDA_TRY(cudaMemcpyAsync(&s->d_sc->switching, &sw, sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *launches += 6 + (s->v.deferred ? 1 : s->m);
    return HBICG_OK;
}

/* A fused solve paused with a full basis (scalars in h_sc): form x_j and
 * p_j, restart the basis (the reset lets the solve run on) and note the last
 * iteration the flush covered. */
static int fused_pause_flush(hbicg_solver *s, int *k_flushed, int *launches, int *flushes, double *flush_ms) {
    cudaStream_t st = s->ctx->stream;
    hbk_scalars *h = s->ctx->h_sc;
    int rc = ensure_pmat(s);
    if (rc) return rc;
    float t = 0.f;
    CUDA_TRY(cudaEventRecord(s->ctx->evf0, st));
    rc = do_flush(s, 1, h->slots, *k_flushed, launches);
    if (rc) return rc;
    *k_flushed = h->k - 1;
    if (s->early_x && (rc = early_copies(s, *k_flushed, launches))) return rc;
    CUDA_TRY(cudaEventRecord(s->ctx->evf1, st));
    CUDA_TRY(cudaEventSynchronize(s->ctx->evf1));
    CUDA_TRY(cudaEventElapsedTime(&t, s->ctx->evf0, s->ctx->evf1));
    *flush_ms += t;
    (*flushes)++;
    return HBICG_OK;
}

/* The end of a fused solve whose iterations are over (h_sc holds its
 * scalars): in the deferred mode the last flush and x_j back to rows; the
 * final scalars in h_sc. */
static int fused_tail(hbicg_solver *s, int k_flushed, int *launches, double *flush_ms) {
    cudaStream_t st = s->ctx->stream;
    hbk_scalars *h = s->ctx->h_sc;
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

/* params.use_graph = 3: the whole solve as one persistent cooperative launch
 * of the shared-launch kernel (hbk_group_run) with this one family, in
 * rounds of one basis block in the deferred mode; its rows are cut into
 * virtual blocks so that about two per SM exist (256..1024 rows each).
 * Measured on GB300 it does not beat the graphs of the default: 5.3 against
 * 5.0 ms on the 32^3 family, 10.3 against 8.4 ms at 48^3, 15.9 against
 * 15.2 ms at 64^3 (deferred): a step's own latency, not the kernel boundary,
 * sets an iteration's length at these sizes, and a grid barrier costs about
 * what a boundary inside a graph does. */
static int run_persistent(hbicg_solver *s, int *launches, int *flushes, double *flush_ms) {
    cudaStream_t st = s->ctx->stream;
    hbk_scalars *h = s->ctx->h_sc;
    const unsigned n = s->A->k.n;
    const unsigned want = (n + 2u * (unsigned)hbk_device_sm_count() - 1u) / (2u * (unsigned)hbk_device_sm_count());
    const unsigned rows = want <= 256u ? 256u : (want >= 1024u ? 1024u : (want + 255u) / 256u * 256u);
    const size_t bytes = hbk_group_ws_bytes(1, &s->v, rows);
    void *ws = NULL;
    int rc = HBICG_OK, k_flushed = 0;
    CUDA_TRY(pool_alloc(&ws, bytes, st));
    for (int round = 0;; ++round) {
        if (round > s->kcap + 64) {
            set_msg("persistent launch: no progress after %d rounds", round);
            rc = HBICG_E_TIMEOUT;
            break;
        }
        int err = 0;
        const int e = hbk_group_run(1, &s->A->k, &s->v, &s->sh, s->kcap, 0, rows, ws, bytes, &err, st);
        ++*launches;
        if (e) {
            set_msg("persistent launch: %s", hbk_error_string(e));
            rc = HBICG_E_CUDA;
            break;
        }
        if (err) {
            set_msg("persistent launch: %s",
                    err == HBK_GROUP_ERR_WAIT ? "a grid barrier's wait timed out" : "the iteration cap was reached");
            rc = HBICG_E_TIMEOUT;
            break;
        }
        cudaError_t ce = cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, st);
        if (!ce) ce = cudaStreamSynchronize(st);
        if (ce) {
            set_msg("persistent launch: %s", cudaGetErrorString(ce));
            rc = HBICG_E_CUDA;
            break;
        }
        if (!(h->finished && (h->status & HBK_ST_BASIS_FULL) && !(h->status & HBK_ST_BREAKDOWN))) break;
        if ((rc = fused_pause_flush(s, &k_flushed, launches, flushes, flush_ms)) != HBICG_OK) break;
    }
    hbicg__dev_free(ws, st);
    if (rc) return rc;
    return fused_tail(s, k_flushed, launches, flush_ms);
}

static int run_fused(hbicg_solver *s, int seed, int *launches, int *flushes, double *flush_ms) {
    cudaStream_t st = s->ctx->stream;
    hbk_scalars *h = s->ctx->h_sc;
    int rc0 = fused_init(s, seed, launches);
    if (rc0) return rc0;
    if (s->p.use_graph == 3 && s->A->k.fmt == HBK_FMT_SELL && s->m > 0) return run_persistent(s, launches, flushes, flush_ms);
    const int use_graph = s->p.use_graph;
    /* every launch of a chunk advances k by chunk unless the solve ends or
     * the basis pauses it; bound the host loop all the same */
    long guard = 0;
    const long guard_max = 4L * s->kcap / s->chunk + 64;
    int k_flushed = 0; /* last iteration covered by a flush */
    int loops_seen = 0; /* loop-graph bodies counted so far (k_init zeroes the device count) */
    for (;;) {
        if (++guard > guard_max) {
            set_msg("fused loop made no progress after %ld chunks", guard_max);
            return HBICG_E_TIMEOUT;
        }
        int looped = 0;
        if (use_graph) {
            if (!s->graph) {
                int rc = capture_graph(s);
                if (rc) return rc;
            }
            CUDA_TRY(cudaGraphLaunch(s->graph, st));
            looped = s->graph_loop;
        } else {
            for (int i = 0; i < s->chunk; i++) HBK_TRY(hbk_fused_iteration(&s->A->k, &s->v, &s->sh, st));
        }
        CUDA_TRY(cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (looped) { /* every body: a chunk of iterations' kernels and the condition kernel */
            *launches += (h->loops - loops_seen) * (s->chunk * s->launches_per_iter + 1);
            loops_seen = h->loops;
        } else {
            *launches += s->chunk * s->launches_per_iter;
        }
        if (!h->finished) continue;
        if ((h->status & HBK_ST_BASIS_FULL) && !(h->status & HBK_ST_BREAKDOWN)) {
            int rc = fused_pause_flush(s, &k_flushed, launches, flushes, flush_ms);
            if (rc) return rc;
            continue;
        }
        break;
    }
    return fused_tail(s, k_flushed, launches, flush_ms);
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

/* One solve in three steps: run_begin (inputs, host scratch, set-up),
 * the iterations, run_end (corrections, outputs, statistics).  A batch runs
 * the iterations of many solves in one launch between the steps
 * (hbicg__group_solve). */
typedef struct {
    int seed, in_where, out_where;
    double *x, *r_out;
    hbicg_stats *stats;
    touch_t touch;
    run_host_t hb;
    int k, n_sw, final_seed, status, launches, flushes;
    double flush_ms;
    const double *r_final;
    double shared_ms; /* >= 0: the iterations ran in a launch shared with other solves, this long */
} run_t;

static void run_release(hbicg_solver *s, run_t *r);
static int run_begin(hbicg_solver *s, const double *b, const double *sigma, run_t *r);
static int run_iterate(hbicg_solver *s, run_t *r);
static int run_end(hbicg_solver *s, run_t *r, int rc);

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

static void run_init(run_t *r, int seed, int in_where, double *x, double *r_out, int out_where, hbicg_stats *stats) {
    memset(r, 0, sizeof *r);
    r->seed = seed;
    r->in_where = in_where;
    r->x = x;
    r->r_out = r_out;
    r->out_where = out_where;
    r->stats = stats;
    r->shared_ms = -1.0;
}

int hbicg_solver_run(hbicg_solver *s, const double *b, const double *sigma, int seed, int in_where, double *x,
                     double *r_out, int out_where, hbicg_stats *stats) {
    run_t r;
    run_init(&r, seed, in_where, x, r_out, out_where, stats);
    int rc = run_begin(s, b, sigma, &r);
    if (rc == HBICG_OK) rc = run_end(s, &r, run_iterate(s, &r));
    run_release(s, &r);
    return rc;
}

/* the page-touching helper is joined, and the host scratch freed, on every
 * return path of the solve */
static void run_release(hbicg_solver *s, run_t *r) {
    touch_join(&r->touch);
    run_host_free(&r->hb);
    /* no copy into the caller's buffer outlives the call, whatever path returned */
    if (s->early_pending) cudaStreamSynchronize(s->ctx->cstream);
    s->early_x = NULL;
    s->early_pending = 0;
    free(s->early);
    s->early = NULL;
}

static int run_begin(hbicg_solver *s, const double *b, const double *sigma, run_t *r) {
    const int seed = r->seed, in_where = r->in_where, out_where = r->out_where;
    double *x = r->x, *r_out = r->r_out;
    touch_t *touch = &r->touch;
    run_host_t *hb = &r->hb;
    hbicg_context *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const unsigned n = s->A->k.n;
    const int m = s->m;
    if (m > 0 && (seed < 0 || seed >= m)) {
        set_msg("seed %d out of range [0, %d)", seed, m);
        return HBICG_E_ARG;
    }
    const enum cudaMemcpyKind kin = in_where == HBICG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
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
    s->flush_bytes = 0.0;
    r->k = 1;
    r->final_seed = seed;
    r->status = HBICG_OK;
    return HBICG_OK;
}

/* after the fused iterations: scalars in the context's host copy (h_sc) */
static int fused_collect(hbicg_solver *s, run_t *r) {
    cudaStream_t st = s->ctx->stream;
    const int m = s->m;
    hbk_scalars *h = s->ctx->h_sc;
    r->k = h->k;
    r->n_sw = h->n_sw;
    r->final_seed = h->seed;
    if (h->status & (HBK_ST_BREAKDOWN | HBK_ST_SHIFT_FAIL)) r->status = HBICG_E_BREAKDOWN;
    if (m > 0) {
        CUDA_TRY(cudaMemcpyAsync(r->hb.conv, s->sh.conv_k, sizeof(int) * m, cudaMemcpyDeviceToHost, st));
        int nl = r->n_sw < m ? r->n_sw : m;
        if (nl) {
            CUDA_TRY(cudaMemcpyAsync(r->hb.sw_k, s->sh.sw_k, sizeof(int) * nl, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaMemcpyAsync(r->hb.sw_seed, s->sh.sw_seed, sizeof(int) * nl, cudaMemcpyDeviceToHost, st));
        }
    }
    CUDA_TRY(cudaMemcpyAsync(r->hb.act, s->sh.act_hist, sizeof(int) * ((size_t)s->kcap + 1), cudaMemcpyDeviceToHost, st));
    r->r_final = s->v.deferred ? s->v.V + (size_t)h->slot_r_old * s->ld : s->v.rbuf[(h->k - 1) & 1];
    return HBICG_OK;
}

static int run_iterate(hbicg_solver *s, run_t *r) {
    const int seed = r->seed;
    int *act = r->hb.act, *sw_k = r->hb.sw_k, *sw_seed = r->hb.sw_seed, *conv = r->hb.conv;
    const double *h_sigma = r->hb.h_sigma;
    int rc = HBICG_OK;
    if (s->p.form == HBICG_FORM_PLAIN) {
        plain_out o;
        memset(&o, 0, sizeof o);
        o.sw_k = sw_k;
        o.sw_seed = sw_seed;
        o.conv_k = conv;
        o.act = act;
        rc = run_plain(s, h_sigma, seed, &o);
        r->k = o.k;
        r->n_sw = o.n_sw;
        r->final_seed = o.final_seed;
        r->launches = o.launches;
        if (rc == HBICG_E_BREAKDOWN) {
            r->status = rc;
            rc = HBICG_OK;
        }
        r->r_final = s->d_r;
    } else {
        rc = run_fused(s, seed, &r->launches, &r->flushes, &r->flush_ms);
        if (rc == HBICG_OK) rc = fused_collect(s, r);
    }
    return rc;
}

static int run_end(hbicg_solver *s, run_t *r, int rc) {
    hbicg_context *ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const unsigned n = s->A->k.n;
    const int m = s->m;
    const int out_where = r->out_where;
    double *x = r->x, *r_out = r->r_out;
    hbicg_stats *stats = r->stats;
    touch_t *touch = &r->touch;
    run_host_t *hb = &r->hb;
    int *act = hb->act, *sw_k = hb->sw_k, *sw_seed = hb->sw_seed, *conv = hb->conv;
    const double *h_sigma = hb->h_sigma;
    const enum cudaMemcpyKind kout = out_where == HBICG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const int k = r->k, n_sw = r->n_sw, final_seed = r->final_seed;
    int status = r->status;
    const double *r_final = r->r_final;
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
        if (r->shared_ms >= 0.0) ms = (float)r->shared_ms;
        else cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        stats->k = k;
        stats->status = rc ? rc : status;
        stats->n_switches = n_sw;
        stats->final_seed = final_seed;
        stats->shift_mode = s->mode;
        stats->basis_flushes = r->flushes;
        stats->launches = r->launches;
        stats->refined_shifts = refined;
        stats->solve_ms = ms;
        stats->flush_ms = r->flush_ms;
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

/* ------------------------------------------------------------------------ */
/* many solves, one launch */

int hbicg__group_eligible(const hbicg_solver *s) {
    return s && s->p.form == HBICG_FORM_FUSED && s->A->k.fmt == HBK_FMT_SELL && s->m > 0;
}

/* Solves of many families whose iterations run in one persistent launch
 * (hbk_group_run).  hbicg__group_add does one solve's first step (run_begin
 * and the fused initialisation, on the solver's own context and stream) and
 * registers it; hbicg__group_launch runs every registered family's iterations
 * in one cooperative launch on the group's own high-priority stream and
 * waits for it; hbicg__group_finish does a family's last step (run_end:
 * corrections, outputs, statistics) on its own stream.  Adds (and finishes)
 * of families on different contexts may run on different host threads; a
 * context's families are finished one after another (they share its pinned
 * scalars).  stats.solve_ms is the shared launch's time and stats.launches
 * counts it once. */
#define GROUP_MSG 192
struct hbicg__group {
    pthread_mutex_t lock;
    int cap, n, max_ctas, lrc, rounds;
    double ms;
    cudaStream_t stream;
    hbicg_solver **S;
    run_t *R;
    int *rc, *in;
    int *k_flushed; /* deferred mode: last iteration the family's previous flush covered */
    int *itrc;      /* a family's own failure between rounds (a flush) */
    /* what the failing call reported, for failures that happen on another
     * thread than the family's finish: a family's set-up or its flush between
     * rounds (per slot), and the launch itself */
    char (*msg)[GROUP_MSG];
    char lmsg[GROUP_MSG];
};

static void group_keep(char *dst) {
    strncpy(dst, hbicg_last_message(), GROUP_MSG - 1);
    dst[GROUP_MSG - 1] = 0;
}

hbicg__group *hbicg__group_new(int cap, int max_ctas) {
    hbicg__group *g = calloc(1, sizeof *g);
    if (!g) return NULL;
    int lo = 0, hi = 0;
    g->cap = cap > 0 ? cap : 1;
    g->max_ctas = max_ctas;
    g->S = calloc((size_t)g->cap, sizeof *g->S);
    g->R = calloc((size_t)g->cap, sizeof *g->R);
    g->rc = calloc((size_t)g->cap, sizeof *g->rc);
    g->in = calloc((size_t)g->cap, sizeof *g->in);
    g->k_flushed = calloc((size_t)g->cap, sizeof *g->k_flushed);
    g->itrc = calloc((size_t)g->cap, sizeof *g->itrc);
    g->msg = calloc((size_t)g->cap, sizeof *g->msg);
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (!e) e = cudaStreamCreateWithPriority(&g->stream, cudaStreamNonBlocking, hi);
    if (!g->S || !g->R || !g->rc || !g->in || !g->k_flushed || !g->itrc || !g->msg || e) {
        if (!e) cudaStreamDestroy(g->stream);
        free(g->S);
        free(g->R);
        free(g->rc);
        free(g->in);
        free(g->k_flushed);
        free(g->itrc);
        free(g->msg);
        free(g);
        return NULL;
    }
    pthread_mutex_init(&g->lock, NULL);
    return g;
}

void hbicg__group_free(hbicg__group *g) {
    if (!g) return;
    cudaStreamSynchronize(g->stream);
    cudaStreamDestroy(g->stream);
    pthread_mutex_destroy(&g->lock);
    free(g->S);
    free(g->R);
    free(g->rc);
    free(g->in);
    free(g->k_flushed);
    free(g->itrc);
    free(g->msg);
    free(g);
}

int hbicg__group_add(hbicg__group *g, hbicg_solver *s, const double *b, const double *sigma, int seed, double *x,
                     hbicg_stats *st) {
    pthread_mutex_lock(&g->lock);
    const int slot = g->n < g->cap ? g->n++ : -1;
    pthread_mutex_unlock(&g->lock);
    if (slot < 0) return -1;
    run_t *r = &g->R[slot];
    run_init(r, seed, HBICG_HOST, x, NULL, HBICG_HOST, st);
    g->S[slot] = s;
    int rc = hbicg__group_eligible(s) ? HBICG_OK : HBICG_E_ARG;
    if (rc) set_msg("a solver that is not fused and SELL-32 cannot join the shared launch");
    if (rc == HBICG_OK) rc = run_begin(s, b, sigma, r);
    if (rc == HBICG_OK) rc = fused_init(s, seed, &r->launches);
    g->rc[slot] = rc;
    g->in[slot] = rc == HBICG_OK;
    if (rc) group_keep(g->msg[slot]);
    return slot;
}

/* Rounds of the shared launch: each runs the iterations of every family
 * still going until each has stopped or paused with a full basis (deferred
 * mode); the paused ones are flushed (their own stream) and run on in the
 * next round. */
int hbicg__group_launch(hbicg__group *g) {
    int err = 0, lrc = HBICG_OK, rounds = 0;
    const int n = g->n;
    hbk_matrix *A = calloc((size_t)n + 1, sizeof(hbk_matrix));
    hbk_vectors *V = calloc((size_t)n + 1, sizeof(hbk_vectors));
    hbk_shifts *H = calloc((size_t)n + 1, sizeof(hbk_shifts));
    int *idx = calloc((size_t)n + 1, sizeof(int)), *run = calloc((size_t)n + 1, sizeof(int));
    void *ws = NULL;
    size_t bytes = 0;
    cudaEvent_t e0 = NULL, e1 = NULL;
    double total_ms = 0.0;
    int kmax = 0;
    if (!A || !V || !H || !idx || !run) {
        lrc = HBICG_E_NOMEM;
        goto out;
    }
    for (int f = 0, q = 0; f < n; ++f) {
        run[f] = g->in[f];
        if (!run[f]) continue;
        V[q++] = g->S[f]->v;
        if (g->S[f]->kcap > kmax) kmax = g->S[f]->kcap;
        bytes = hbk_group_ws_bytes(q, V, 0); /* the first round takes every family: the most virtual blocks */
    }
    if (!bytes) goto out;
    if (pool_alloc(&ws, bytes, g->stream) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        lrc = HBICG_E_NOMEM;
        goto out;
    }
    /* a round advances every running family by a basis block or to its end */
    for (;; ++rounds) {
        int ng = 0, cap = 0, resumed = 0;
        for (int f = 0; f < n; ++f) {
            if (!run[f]) continue;
            const hbicg_solver *s = g->S[f];
            A[ng] = s->A->k;
            V[ng] = s->v;
            H[ng] = s->sh;
            idx[ng] = f;
            if (s->kcap > cap) cap = s->kcap;
            ++ng;
        }
        if (!ng) break;
        if (rounds > kmax + 64) {
            set_msg("shared launch: no family finished after %d rounds", rounds);
            lrc = HBICG_E_TIMEOUT;
            break;
        }
        float ms = 0.f;
        cudaEventRecord(e0, g->stream);
        const int e = hbk_group_run(ng, A, V, H, cap, g->max_ctas, 0, ws, bytes, &err, g->stream);
        cudaEventRecord(e1, g->stream);
        if (e || cudaStreamSynchronize(g->stream) != cudaSuccess) {
            set_msg("shared launch: %s", hbk_error_string(e ? e : (int)cudaGetLastError()));
            lrc = HBICG_E_CUDA;
            break;
        }
        if (err) {
            set_msg("shared launch: %s",
                    err == HBK_GROUP_ERR_WAIT ? "a grid barrier's wait timed out" : "the iteration cap was reached");
            lrc = HBICG_E_TIMEOUT;
            break;
        }
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        for (int q = 0; q < ng; ++q) {
            const int f = idx[q];
            hbicg_solver *s = g->S[f];
            run_t *r = &g->R[f];
            hbk_scalars *h = s->ctx->h_sc;
            r->launches += 1;
            cudaError_t ce = cudaMemcpyAsync(h, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost, s->ctx->stream);
            if (!ce) ce = cudaStreamSynchronize(s->ctx->stream);
            if (ce) {
                set_msg("shared launch: %s", cudaGetErrorString(ce));
                g->itrc[f] = HBICG_E_CUDA;
                group_keep(g->msg[f]);
                run[f] = 0;
            } else if (h->finished && (h->status & HBK_ST_BASIS_FULL) && !(h->status & HBK_ST_BREAKDOWN)) {
                g->itrc[f] = fused_pause_flush(s, &g->k_flushed[f], &r->launches, &r->flushes, &r->flush_ms);
                if (g->itrc[f]) group_keep(g->msg[f]);
                run[f] = g->itrc[f] == HBICG_OK;
                resumed += run[f];
            } else {
                run[f] = 0; /* converged, at max_iter or broken down */
            }
        }
        if (!resumed) {
            ++rounds;
            break;
        }
    }
out:
    if (ws) hbicg__dev_free(ws, g->stream);
    cudaStreamSynchronize(g->stream);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    free(A);
    free(V);
    free(H);
    free(idx);
    free(run);
    g->lrc = lrc;
    if (lrc) group_keep(g->lmsg);
    g->ms = total_ms;
    g->rounds = rounds;
    return lrc;
}

int hbicg__group_finish(hbicg__group *g, int slot) {
    if (slot < 0 || slot >= g->n) return HBICG_E_ARG;
    hbicg_solver *s = g->S[slot];
    run_t *r = &g->R[slot];
    int rc = g->rc[slot];
    if (rc) set_msg("%s", g->msg[slot]); /* its set-up failed */
    if (g->in[slot]) {
        int it = g->lrc != HBICG_OK ? g->lrc : g->itrc[slot];
        if (it != HBICG_OK) set_msg("%s", g->lrc != HBICG_OK ? g->lmsg : g->msg[slot]);
        if (it == HBICG_OK) { /* the final flush reads this family's scalars (its context's copy may hold another's) */
            cudaError_t ce = cudaMemcpyAsync(s->ctx->h_sc, s->d_sc, sizeof(hbk_scalars), cudaMemcpyDeviceToHost,
                                             s->ctx->stream);
            if (!ce) ce = cudaStreamSynchronize(s->ctx->stream);
            if (ce) {
                set_msg("shared launch: %s", cudaGetErrorString(ce));
                it = HBICG_E_CUDA;
            }
        }
        if (it == HBICG_OK) it = fused_tail(s, g->k_flushed[slot], &r->launches, &r->flush_ms);
        if (it == HBICG_OK) it = fused_collect(s, r);
        r->shared_ms = g->ms;
        rc = run_end(s, r, it);
    }
    run_release(s, r);
    g->rc[slot] = rc;
    return rc;
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
