/* Batched families: many independent shifted systems (A_f + sigma_fj I) x = b_f
 * solved on one GPU.
 *
 * The reference solves one family per program run and sweeps seeds or
 * matrices with hard-coded loops in its drivers (src/main_seed_diff.c:113-155,
 * src/main_repeat.c).  A family of n = 10^4..5*10^5 unknowns fills only a part
 * of GB300 (one SpMV is a few hundred blocks, one iteration is eight short
 * kernels and a few scalar steps), so here a pool of host workers, each with
 * its own context and CUDA stream, takes families from a shared queue (largest
 * nnz * m first) and runs them concurrently: the GPU interleaves the kernels of
 * several families.  Each family is a complete reference-semantics solve
 * (hbicg_solver_run), with the optional SpMV-form autotuner in front.
 *
 * Small families (incremental shift mode: n m < 2^21 with the automatic mode)
 * are latency-bound when each runs its own short kernels: they instead go to
 * a few host threads that set all of them up and run all their iterations in
 * ONE persistent cooperative launch (hbicg__group_*, hbk_group_run), while
 * the workers take the larger families.  With opts.persistent = 2 every
 * family goes to the shared launch (those in the deferred shift mode pause
 * there at each full basis; the host flushes them between rounds).
 * Failures are per family (status), never global. */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "hbicg.h"
#include "host_internal.h"

typedef struct {
    hbicg_family *fams;
    const int *order;
    int count;
    const hbicg_params *p;
    const char *cache;
    int next;    /* queue position (atomic) */
    char *msgs;  /* [families][FAIL_MSG]: what a failing family's call reported */
} batch_t;

/* The message of a family whose status is not OK: its thread's
 * hbicg_last_message right after the failing call, kept per family so that
 * the batch can hand the first failure's message to its caller. */
#define FAIL_MSG 192
static void keep_msg(char *msgs, const hbicg_family *base, const hbicg_family *f) {
    if (!msgs || f->status == HBICG_OK) return;
    char *dst = msgs + (size_t)(f - base) * FAIL_MSG;
    strncpy(dst, hbicg_last_message(), FAIL_MSG - 1);
    dst[FAIL_MSG - 1] = 0;
}

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void solve_one(hbicg_context *ctx, hbicg_family *f, const hbicg_params *p, const char *cache) {
    const double t0 = now_ms();
    hbicg_matrix *A = NULL;
    hbicg_solver *s = NULL;
    f->status = hbicg_matrix_create(ctx, f->n, f->nnz, f->ptr, f->col, f->val, HBICG_HOST, &A);
    if (f->status == HBICG_OK && f->autotune) f->status = hbicg_matrix_autotune(A, cache, NULL, NULL, NULL);
    if (f->status == HBICG_OK) {
        f->spmv_format = hbicg_matrix_format(A);
        f->status = hbicg_solver_create(ctx, A, f->m, p, &s);
    }
    if (f->status == HBICG_OK) {
        hbicg_stats st;
        memset(&st, 0, sizeof st);
        st.true_residual = f->true_residual;
        f->status = hbicg_solver_run(s, f->b, f->sigma, f->seed, HBICG_HOST, f->x, f->r, HBICG_HOST, &st);
        f->k = st.k;
        f->n_switches = st.n_switches;
        f->final_seed = st.final_seed;
        f->solve_ms = st.solve_ms;
        f->max_true_residual = st.max_true_residual;
    }
    hbicg_solver_destroy(s);
    hbicg_matrix_destroy(A);
    f->wall_ms = now_ms() - t0;
}

static void family_stats(hbicg_family *f, const hbicg_stats *st) {
    f->k = st->k;
    f->n_switches = st->n_switches;
    f->final_seed = st->final_seed;
    f->solve_ms = st->solve_ms;
    f->max_true_residual = st->max_true_residual;
}

/* Families of one persistent launch (see the file comment).  Up to
 * GROUP_THREADS host threads, each with its own high-priority context, take
 * the families from a shared index and set them up (matrix, solver, the
 * solve's first step: hbicg__group_add); once all have, thread 0 signals the
 * batch (which then starts its workers) and runs the one launch; then every
 * thread finishes its own families (hbicg__group_finish). */
#define GROUP_THREADS 4
typedef struct {
    hbicg_family *fams;
    const int *idx;
    int count;
    const hbicg_params *p;
    hbicg__group *g;
    int next;              /* shared index (atomic) */
    int nthreads;          /* threads taking part (lowered when one fails to start) */
    int arrived[2];        /* threads at each of the two meeting points */
    int setup_done;
    pthread_mutex_t m;
    pthread_cond_t cv;
    int *slot;             /* [count] slot in g, -1: solved on its own */
    hbicg_stats *st;       /* [count] */
    hbicg_matrix **A;      /* [count] */
    hbicg_solver **S;      /* [count] */
    char *msgs;            /* as in batch_t, indexed by family */
} group_t;

typedef struct {
    group_t *G;
    int tid;
} part_t;

static void meet(group_t *G, int point) {
    pthread_mutex_lock(&G->m);
    G->arrived[point]++;
    pthread_cond_broadcast(&G->cv);
    while (G->arrived[point] < G->nthreads) pthread_cond_wait(&G->cv, &G->m);
    pthread_mutex_unlock(&G->m);
}

static void *group_part(void *arg) {
    part_t *pa = arg;
    group_t *G = pa->G;
    const double t0 = now_ms();
    hbicg_context *ctx = NULL;
    const int crc = hbicg__context_create_prio(&ctx, 1);
    int *mine = malloc(sizeof(int) * (size_t)(G->count > 0 ? G->count : 1)), nm = 0;
    for (;;) {
        const int i = __atomic_fetch_add(&G->next, 1, __ATOMIC_RELAXED);
        if (i >= G->count) break;
        hbicg_family *f = &G->fams[G->idx[i]];
        G->slot[i] = -1;
        if (crc != HBICG_OK || !mine) {
            f->status = crc != HBICG_OK ? crc : HBICG_E_NOMEM;
            keep_msg(G->msgs, G->fams, f);
            continue;
        }
        mine[nm++] = i;
        f->status = hbicg_matrix_create(ctx, f->n, f->nnz, f->ptr, f->col, f->val, HBICG_HOST, &G->A[i]);
        if (f->status == HBICG_OK) {
            f->spmv_format = hbicg_matrix_format(G->A[i]);
            f->status = hbicg_solver_create(ctx, G->A[i], f->m, G->p, &G->S[i]);
        }
        if (f->status != HBICG_OK) {
            keep_msg(G->msgs, G->fams, f);
            continue;
        }
        G->st[i].true_residual = f->true_residual;
        if (hbicg__group_eligible(G->S[i])) {
            G->slot[i] = hbicg__group_add(G->g, G->S[i], f->b, f->sigma, f->seed, f->x, &G->st[i]);
            if (G->slot[i] < 0) { /* no room in the shared launch (not expected) */
                f->status = HBICG_E_ARG;
                hbicg__set_msg("no slot left in the shared persistent launch");
            }
        } else { /* another form after all (e.g. rows too long for SELL-32): a solve of its own */
            f->status = hbicg_solver_run(G->S[i], f->b, f->sigma, f->seed, HBICG_HOST, f->x, f->r, HBICG_HOST,
                                         &G->st[i]);
            family_stats(f, &G->st[i]);
        }
        keep_msg(G->msgs, G->fams, f);
    }
    meet(G, 0);
    if (pa->tid == 0) {
        pthread_mutex_lock(&G->m);
        G->setup_done = 1;
        pthread_cond_broadcast(&G->cv);
        pthread_mutex_unlock(&G->m);
        hbicg__group_launch(G->g);
    }
    meet(G, 1);
    for (int q = 0; q < nm; ++q) {
        const int i = mine[q];
        hbicg_family *f = &G->fams[G->idx[i]];
        if (G->slot[i] >= 0) {
            f->status = hbicg__group_finish(G->g, G->slot[i]);
            family_stats(f, &G->st[i]);
            keep_msg(G->msgs, G->fams, f);
        }
        hbicg_solver_destroy(G->S[i]);
        hbicg_matrix_destroy(G->A[i]);
        f->wall_ms = now_ms() - t0;
    }
    if (ctx) hbicg_context_destroy(ctx);
    free(mine);
    return NULL;
}

static void *worker(void *arg) {
    batch_t *b = arg;
    hbicg_context *ctx = NULL;
    int rc = hbicg_context_create(&ctx);
    for (;;) {
        const int i = __atomic_fetch_add(&b->next, 1, __ATOMIC_RELAXED);
        if (i >= b->count) break;
        hbicg_family *f = &b->fams[b->order[i]];
        if (rc != HBICG_OK) {
            f->status = rc;
            keep_msg(b->msgs, b->fams, f);
            continue;
        }
        solve_one(ctx, f, b->p, b->cache);
        keep_msg(b->msgs, b->fams, f);
    }
    if (ctx) hbicg_context_destroy(ctx);
    return NULL;
}

static const hbicg_family *g_sort_base;
static int by_cost_desc(const void *x, const void *y) {
    const hbicg_family *a = &g_sort_base[*(const int *)x], *b = &g_sort_base[*(const int *)y];
    const double ca = (double)a->nnz * (a->m + 2), cb = (double)b->nnz * (b->m + 2);
    if (ca != cb) return ca > cb ? -1 : 1;
    return *(const int *)x - *(const int *)y;
}

void hbicg_batch_opts_default(hbicg_batch_opts *o) {
    memset(o, 0, sizeof *o);
    o->workers = 8;
    o->persistent = 1;
}

int hbicg_batch_solve(hbicg_family *fams, int count, const hbicg_params *p, int workers, const char *autotune_cache,
                      double *wall_ms) {
    hbicg_batch_opts o;
    hbicg_batch_opts_default(&o);
    o.workers = workers;
    o.autotune_cache = autotune_cache;
    return hbicg_batch_solve_opts(fams, count, p, &o, wall_ms);
}

int hbicg_batch_solve_opts(hbicg_family *fams, int count, const hbicg_params *p, const hbicg_batch_opts *opts,
                           double *wall_ms) {
    if (count < 0 || (count && !fams) || !opts) return HBICG_E_ARG;
    const double t0 = now_ms();
    hbicg_params def;
    if (!p) {
        hbicg_params_default(&def);
        p = &def;
    }
    int workers = opts->workers;
    const char *autotune_cache = opts->autotune_cache;
    int *order = malloc(sizeof(int) * (size_t)(count > 0 ? count : 1));
    int *grp = malloc(sizeof(int) * (size_t)(count > 0 ? count : 1));
    char *msgs = calloc((size_t)(count > 0 ? count : 1), FAIL_MSG); /* optional: NULL keeps no messages */
    if (!order || !grp) {
        free(order);
        free(grp);
        free(msgs);
        return HBICG_E_NOMEM;
    }
    for (int i = 0; i < count; i++) {
        order[i] = i;
        fams[i].status = -1;
    }
    static pthread_mutex_t sort_lock = PTHREAD_MUTEX_INITIALIZER;
    pthread_mutex_lock(&sort_lock);
    g_sort_base = fams;
    qsort(order, (size_t)count, sizeof(int), by_cost_desc);
    pthread_mutex_unlock(&sort_lock);
    /* the families of the persistent launch leave the workers' queue */
    int ng = 0, nw = 0;
    for (int i = 0; i < count; i++) {
        const hbicg_family *f = &fams[order[i]];
        const int small = opts->persistent && p->form == HBICG_FORM_FUSED && !f->autotune && !f->r && f->m > 0 &&
                          (opts->persistent >= 2 ||
                           hbicg__shift_mode_for(p, f->n, f->m) == HBICG_SHIFTS_INCREMENTAL);
        if (small) grp[ng++] = order[i];
        else order[nw++] = order[i];
    }
    count = nw;
    group_t G;
    memset(&G, 0, sizeof G);
    part_t parts[GROUP_THREADS];
    pthread_t gth[GROUP_THREADS];
    int g_started = 0;
    if (ng) {
        G.fams = fams;
        G.idx = grp;
        G.count = ng;
        G.p = p;
        G.msgs = msgs;
        G.g = hbicg__group_new(ng, opts->persistent_ctas);
        G.slot = malloc(sizeof(int) * (size_t)ng);
        G.st = calloc((size_t)ng, sizeof(hbicg_stats));
        G.A = calloc((size_t)ng, sizeof(hbicg_matrix *));
        G.S = calloc((size_t)ng, sizeof(hbicg_solver *));
        pthread_mutex_init(&G.m, NULL);
        pthread_cond_init(&G.cv, NULL);
        if (!G.g || !G.slot || !G.st || !G.A || !G.S) { /* no shared launch: the workers take them */
            for (int i = 0; i < ng; i++) order[nw++] = grp[i];
            count = nw;
            ng = 0;
        } else {
            const int want = ng < GROUP_THREADS ? ng : GROUP_THREADS;
            G.nthreads = want;
            for (int t = 0; t < want; t++) {
                parts[t].G = &G;
                parts[t].tid = g_started;
                if (pthread_create(&gth[g_started], NULL, group_part, &parts[t]) == 0) {
                    g_started++;
                } else {
                    pthread_mutex_lock(&G.m);
                    G.nthreads--;
                    pthread_cond_broadcast(&G.cv);
                    pthread_mutex_unlock(&G.m);
                }
            }
            if (!g_started) { /* no thread: the whole group here, before the workers */
                G.nthreads = 1;
                parts[0].G = &G;
                parts[0].tid = 0;
                group_part(&parts[0]);
            } else { /* the workers start once the group is set up (its many short steps then run on an idle GPU) */
                pthread_mutex_lock(&G.m);
                while (!G.setup_done) pthread_cond_wait(&G.cv, &G.m);
                pthread_mutex_unlock(&G.m);
            }
        }
    }
    if (workers < 1) workers = 8;
    if (workers > count) workers = count > 0 ? count : 1;
    if (workers > 64) workers = 64;
    batch_t b = {fams, order, count, p, autotune_cache, 0, msgs};
    pthread_t th[64];
    int started = 0;
    for (int t = 0; t < workers; t++) {
        if (pthread_create(&th[t], NULL, worker, &b) != 0) break;
        started++;
    }
    if (!started && count) worker(&b); /* no threads: run in the caller */
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    for (int t = 0; t < g_started; t++) pthread_join(gth[t], NULL);
    if (G.g) hbicg__group_free(G.g);
    if (G.count) {
        pthread_mutex_destroy(&G.m);
        pthread_cond_destroy(&G.cv);
    }
    free(G.slot);
    free(G.st);
    free(G.A);
    free(G.S);
    count = nw + ng;
    free(order);
    free(grp);
    if (wall_ms) *wall_ms = now_ms() - t0;
    int rc = HBICG_OK;
    for (int i = 0; i < count; i++)
        if (fams[i].status != HBICG_OK) {
            rc = fams[i].status < 0 ? HBICG_E_ARG : fams[i].status;
            if (msgs && msgs[(size_t)i * FAIL_MSG])
                hbicg__set_msg("family %d: %s", i, msgs + (size_t)i * FAIL_MSG);
            else
                hbicg__set_msg("family %d: status %d", i, fams[i].status);
            break;
        }
    free(msgs);
    return rc;
}
