/* Extended C API of the GB300 shifted BiCGStab solver.
 *
 * The reference has no counterpart beyond its three solver entry points
 * (src/solver.h:33-35); this API adds what a library needs around them:
 * run-time parameters instead of compile-time constants (src/solver.h:13-31),
 * status codes instead of exit() (src/solver_dynamic.c:11-14), per-solve
 * statistics (switch log, per-shift convergence iteration, true residuals,
 * timings), device-pointer entry points that keep inputs resident in HBM, and
 * a matrix/solver split so the device CSR, the SpMV schedule, the workspace
 * and the captured CUDA graphs are built once and reused.
 *
 * Threading: one hbicg_context per host thread (each owns a CUDA stream).
 */
#ifndef HBICG_H
#define HBICG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    HBICG_OK = 0,
    HBICG_E_NOT_SQUARE = 1,
    HBICG_E_NO_DIAG = 2,
    HBICG_E_BREAKDOWN = 3, /* (r^,s), (q,y) or a seed scalar became 0, inf or nan (the solve stops), or a
                              non-seed shift's pi_k, 1 - omega_k (sigma_s - sigma_j) or update scalar did
                              (that shift stops at its last finite iterate, the others run to the end) */
    HBICG_E_MAXITER = 4,   /* some shift did not converge within max_iter */
    HBICG_E_CUDA = 5,
    HBICG_E_TIMEOUT = 6,
    HBICG_E_ARG = 7,
    HBICG_E_NOMEM = 8,
    HBICG_E_IO = 9
} hbicg_status;

typedef enum { HBICG_FORM_PLAIN = 0, HBICG_FORM_FUSED = 1 } hbicg_form;

typedef enum {
    HBICG_SHIFTS_AUTO = 0,
    HBICG_SHIFTS_INCREMENTAL = 1, /* x_j, p_j updated every iteration by one multi-shift kernel */
    HBICG_SHIFTS_DEFERRED = 2     /* x_j, p_j kept as coefficients over the seed's Krylov basis */
} hbicg_shift_mode;

typedef enum { HBICG_HOST = 0, HBICG_DEVICE = 1 } hbicg_memory;

typedef struct {
    double tol;            /* relative tolerance on the recursive residual (default 1e-12) */
    int max_iter;          /* default 2000; the loop runs while k < max_iter + 1 */
    int switching;         /* 1 = seed switching (default) */
    int form;              /* hbicg_form, default FUSED */
    int shift_mode;        /* hbicg_shift_mode, default AUTO */
    int use_graph;         /* fused form: 0 = eager launches; 1 = CUDA graphs of graph_chunk iterations, the
                              host checks the scalars after each (default); 2 = one graph whose conditional
                              while node loops over iterations until the solve stops (chunks where the
                              runtime refuses it); 3 = the whole solve as one persistent cooperative launch
                              (grid barriers between the steps; in the deferred mode one launch per basis
                              block, SELL-32 matrices; other forms use 1) */
    int graph_chunk;       /* iterations per graph launch, 0 = automatic */
    double basis_mem_frac; /* deferred mode: share of free device memory for the basis (default 0.6) */
    int true_residuals;    /* compute ||b-(A+sigma_j I)x_j||/||b|| after the solve (default 0) */
    int basis_block;       /* deferred mode: iterations per basis block before x_j, p_j are formed
                              (0 = automatic, 28; < 0 = as long as memory allows) */
    int flush_mode;        /* deferred mode: hbicg_flush_mode (default AUTO) */
    int refine;            /* 1: after the solve, check every shift's true residual
                              ||b - (A + sigma_j I) x_j|| / ||b|| and correct shifts above
                              tol by solving (A + sigma_j I) e = r_j (at most 3 rounds).
                              The recursive residual the reference tests can leave the
                              true one above tol.  Default 1; the reference's entry points
                              (solver.h) use 0 and return the reference's result. */
} hbicg_params;

typedef enum {
    HBICG_FLUSH_AUTO = 0,   /* tensor cores when the basis block fits one K = 64 operand */
    HBICG_FLUSH_FP64 = 1,   /* FP64 CUDA-core kernel */
    HBICG_FLUSH_TENSOR = 2  /* tensor cores (BF16 digit products, FP64-accurate) */
} hbicg_flush_mode;

typedef struct {
    int k;                    /* the reference's return value: iterations + 1 on convergence */
    int status;               /* hbicg_status */
    int n_switches;
    int final_seed;
    int shift_mode;           /* mode actually used */
    int basis_flushes;        /* deferred mode: basis flushes during the solve */
    int launches;             /* kernel launches issued for the solve */
    int refined_shifts;       /* corrections made by params.refine */
    double solve_ms;          /* device time of init + iterations + final flush (CUDA events) */
    double flush_ms;          /* deferred mode: device time of the basis flushes */
    double max_true_residual; /* when params.true_residuals */
    double bytes_algorithmic; /* compulsory HBM bytes of the fused schedule for this solve */
    double flush_bytes;       /* deferred mode: compulsory HBM bytes of the basis flushes (in flush_ms) */
    /* optional caller-owned outputs (NULL to skip) */
    int *switch_k;            /* [m] iteration of each switch */
    int *switch_seed;         /* [m] seed chosen at each switch */
    int *conv_k;              /* [m] iteration at which each shift met the test (0 = never,
                                 -k = broke down at iteration k) */
    int *active_per_iter;     /* [max_iter + 1] non-seed shifts updated at iteration k */
    double *true_residual;    /* [m] */
    double *seed_alpha;       /* [max_iter + 1] the seed's alpha, beta, omega per iteration (as archived) */
    double *seed_beta;
    double *seed_omega;
    double *seed_rr;          /* [max_iter + 1] (r, r) at the end of each iteration */
} hbicg_stats;

typedef struct hbicg_context hbicg_context;
typedef struct hbicg_matrix hbicg_matrix;
typedef struct hbicg_solver hbicg_solver;

void hbicg_params_default(hbicg_params *p);
const char *hbicg_status_string(int status);
/* message of the last failure in this thread (CUDA error text, argument) */
const char *hbicg_last_message(void);

int hbicg_context_create(hbicg_context **ctx);
void hbicg_context_destroy(hbicg_context *ctx);
/* the context's CUDA stream (cudaStream_t) */
void *hbicg_context_stream(hbicg_context *ctx);

/* Square CSR with 32-bit indices; `where` says whether ptr/col/val are host or
 * device pointers (device arrays are used in place, host arrays are copied). */
int hbicg_matrix_create(hbicg_context *ctx, unsigned n, unsigned nnz, const unsigned *ptr, const unsigned *col,
                        const double *val, int where, hbicg_matrix **out);
void hbicg_matrix_destroy(hbicg_matrix *A);
unsigned hbicg_matrix_rows(const hbicg_matrix *A);
unsigned long long hbicg_matrix_nnz(const hbicg_matrix *A);
/* y = A x (+ sigma x); x, y device or host per `where` */
int hbicg_matrix_spmv(hbicg_matrix *A, const double *x, double *y, double sigma, int where);
/* Profiling helper: `iters` back-to-back launches of the SpMV kernel (device
 * x, y) between CUDA events on the context's stream; *ms = mean per launch. */
int hbicg_matrix_time_spmv(hbicg_matrix *A, const double *x, double *y, double sigma, int iters, double *ms);

/* SpMV form of a matrix: CSR row blocks staged in shared memory (TILE);
 * SELL-32, slices of 32 consecutive rows padded to their longest row (rows of
 * at most 64 entries, padding under a third of the nonzeros); HYB, rows of
 * at most 32 entries in SELL-32 slices sorted by length inside windows of 256
 * rows and longer rows one warp each; or MERGE, rows of at most 255 entries in
 * blocks of at most 256 row ends + nonzeros, one warp per block, split evenly
 * among its 32 lanes along the merge path (nonzero-balanced, no copy of the
 * values), longer rows one warp each.  A new matrix takes SELL-32 where it
 * qualifies, else HYB; the autotuner picks among all four. */
typedef enum { HBICG_SPMV_TILE = 0, HBICG_SPMV_SELL = 1, HBICG_SPMV_HYB = 2, HBICG_SPMV_MERGE = 3 } hbicg_spmv_format;
int hbicg_matrix_format(const hbicg_matrix *A);
/* Switch the SpMV form (builds that form's copy if needed; HBICG_E_ARG when a
 * row is too long for SELL-32).  Call before creating solvers on A. */
int hbicg_matrix_set_format(hbicg_matrix *A, int fmt);
/* Autotuner: the pattern's signature (log2 n, longest row, share of rows per
 * power-of-two length class) is looked up in the cache file; if absent, every
 * form the matrix has is timed (10 products each) and the fastest is appended
 * to the cache.  The matrix is left in the chosen form and the copies of the
 * other packed forms are freed.  Cache format (text, one entry per line after
 * a '#' header): "<signature> <tile|sell|hyb> <tile_ms> <packed_ms>", where
 * packed_ms is the SELL-32 time, or the HYB time when HYB was chosen or there
 * is no SELL-32 form.  cache_path NULL: time, no cache.  chosen/tile_ms/sell_ms
 * (the packed time) may be NULL.  Call before creating solvers on A. */
int hbicg_matrix_autotune(hbicg_matrix *A, const char *cache_path, int *chosen, double *tile_ms, double *sell_ms);

/* Coordinate (triplet) matrix in host memory, 0-based, as read from a file. */
typedef struct {
    unsigned rows, cols;
    unsigned long long nnz;
    int field;     /* 0 real, 1 integer, 2 pattern (values 1.0) */
    int symmetry;  /* 0 general, 1 symmetric, 2 skew-symmetric */
    int expanded;  /* mirrored off-diagonal entries appended after the stored ones */
    unsigned *row, *col;
    double *val;
} hbicg_coo;

/* Parallel Matrix Market reader (replaces src/matrix.c:26-94 / src/mmio.c's
 * one-fscanf-per-entry loop): `threads` host threads (0 = all cores), entries
 * in file order, values converted exactly as fscanf("%lg") does.  Symmetric
 * and skew-symmetric files are returned as stored unless expand_symmetric.
 * Errors (I/O, bad banner, bad entry, entry count) return HBICG_E_IO with a
 * message; nothing exits.  Free with hbicg_coo_free. */
int hbicg_mm_read(const char *path, int expand_symmetric, int threads, hbicg_coo *out);
void hbicg_coo_free(hbicg_coo *coo);

/* Square CSR matrix from COO triplets, built on the GPU: entries are ordered
 * by row with the order of entries inside a row kept (the ordering of the
 * reference's coo2csr, src/matrix.c:206-242).  row/col/val are host or device
 * pointers per `where`; indices must be < n (else HBICG_E_ARG). */
int hbicg_matrix_from_coo(hbicg_context *ctx, unsigned n, unsigned nnz, const unsigned *row, const unsigned *col,
                          const double *val, int where, hbicg_matrix **out);
/* Copy the matrix's CSR arrays out (ptr [n+1], col and val [nnz]) to host or
 * device memory per `where`. */
int hbicg_matrix_get_csr(const hbicg_matrix *A, unsigned *ptr, unsigned *col, double *val, int where);
/* hbicg_mm_read + hbicg_matrix_from_coo (the file must be square). */
int hbicg_matrix_load_mm(hbicg_context *ctx, const char *path, int expand_symmetric, hbicg_matrix **out);

/* Workspace for families of m shifts on A (device vectors, scalar state, graphs). */
int hbicg_solver_create(hbicg_context *ctx, hbicg_matrix *A, int m, const hbicg_params *p, hbicg_solver **out);
void hbicg_solver_destroy(hbicg_solver *s);
/* Solve.  b [n], sigma [m] and x [m*n, shift-major, leading dimension n] are
 * host or device pointers per in_where / out_where; r_out [n] (optional)
 * receives the final seed residual.  Returns hbicg_status; stats optional. */
int hbicg_solver_run(hbicg_solver *s, const double *b, const double *sigma, int seed, int in_where, double *x,
                     double *r_out, int out_where, hbicg_stats *stats);

/* True relative residuals ||b - (A + sigma_j I) x_j|| / ||b|| into res[0..m)
 * without allocating anything.  No counterpart in the reference.  For callers
 * that cannot call cudaMalloc where they check a solve (another component owns
 * the device memory budget, a latency-bound loop cannot take cudaMalloc's
 * implicit synchronisation, a host callback may not allocate).  All pointers
 * are device pointers; x is m rows of ldx doubles; work is queued on `stream`
 * (a cudaStream_t, 0 = legacy default) and the call does not wait for it.
 * Scratch is one static device array of about 1 MiB in the library, held by
 * every GPU that loads it until exit: at most HBICG_NOALLOC_MAX_SHIFTS shifts
 * (larger m returns HBICG_E_ARG), and calls that overlap on the GPU race on
 * the shared scratch.  The first call on a device looks the array up with
 * cudaGetSymbolAddress; make it before any stream capture. */
#define HBICG_NOALLOC_MAX_SHIFTS 64
int hbicg_true_residuals_noalloc(hbicg_matrix *A, const double *x, unsigned long long ldx, const double *b,
                                 const double *sigma, int m, double *res, void *stream);

/* Batched families: independent shifted families, each a complete solve with
 * the reference's semantics, run concurrently by `workers` host threads (each
 * with its own context and stream; 0 = 8), largest nnz * m first, so the GPU
 * interleaves the kernels of several small families.  Replaces the
 * reference's hard-coded sweep drivers (src/main_seed_diff.c:113-155).
 * All pointers are host memory.  Per-family status in fams[i].status; the
 * call returns the first failing status (in family order), or HBICG_OK, and
 * hbicg_last_message() on the calling thread then names that family and what
 * its failing call reported.  autotune_cache: path
 * of the SpMV-form cache used by families with autotune set (may be NULL). */
typedef struct {
    /* inputs */
    unsigned n, nnz;
    const unsigned *ptr, *col;
    const double *val;
    const double *b;
    const double *sigma;
    int m, seed;
    int autotune;             /* run hbicg_matrix_autotune before the solve */
    /* outputs */
    double *x;                /* [m*n], shift-major */
    double *r;                /* [n] final seed residual (optional) */
    double *true_residual;    /* [m] when params.true_residuals (optional) */
    int status, k, n_switches, final_seed, spmv_format;
    double solve_ms;          /* device time of the solve */
    double wall_ms;           /* host time of matrix set-up + solve + copies */
    double max_true_residual;
} hbicg_family;
int hbicg_batch_solve(hbicg_family *fams, int count, const hbicg_params *p, int workers, const char *autotune_cache,
                      double *wall_ms);
/* The same with every option.  persistent = 1 (the default of
 * hbicg_batch_solve too): the families that take the incremental shift mode
 * (n m < 2^21 with shift_mode AUTO; no autotune, no residual output) run all
 * their iterations in one persistent launch on the GPU, set up and finished
 * by a few host threads, while the workers take the other families.
 * persistent = 2: every such family whatever its shift mode (deferred-mode
 * families pause in the launch at each full basis and are flushed between
 * rounds of it); 0: every family on the workers. */
typedef struct {
    int workers;                /* host workers for the other families (default 8) */
    int persistent;             /* 0, 1 (default) or 2 */
    int persistent_ctas;        /* CTAs of the persistent launch; 0 = one wave of the GPU */
    const char *autotune_cache; /* as in hbicg_batch_solve */
} hbicg_batch_opts;
void hbicg_batch_opts_default(hbicg_batch_opts *o);
int hbicg_batch_solve_opts(hbicg_family *fams, int count, const hbicg_params *p, const hbicg_batch_opts *opts,
                           double *wall_ms);

/* Adjoint (no counterpart in the reference, which only solves forward).
 * A^T as a new matrix on A's context, built on the GPU (stable by column). */
int hbicg_matrix_transpose(hbicg_matrix *A, hbicg_matrix **At);
/* Gradients from given solutions, all device pointers: X [m][ldx] with
 * (A + sigma_j I) x_j = b, Lam [m][ldl] with (A^T + sigma_j I) lam_j = g_j,
 * weights w [m] (NULL = ones):
 *   dJ_dval[e] = -sum_j w_j lam_j[row e] x_j[col e],  dJ_db = sum_j w_j lam_j,
 *   dJ_dsigma[j] = -w_j lam_j . x_j   (each output may be NULL). */
int hbicg_adjoint_gradients(hbicg_matrix *A, int m, const double *X, unsigned long long ldx, const double *Lam,
                            unsigned long long ldl, const double *w, double *dJ_dval, double *dJ_db,
                            double *dJ_dsigma);
/* J = sum_j w_j c^T x_j and its gradients for a family on A (host pointers
 * in and out; At may be NULL to build A^T here).  One forward family on A
 * and one transposed family on A^T with right-hand side c, same shifts and
 * seed; fwd/adj stats optional; x_out [m*n] optional. */
int hbicg_adjoint(hbicg_matrix *A, hbicg_matrix *At, const double *b, const double *sigma, int m, int seed,
                  const double *w, const double *c, const hbicg_params *p, double *J, double *dJ_dval, double *dJ_db,
                  double *dJ_dsigma, double *x_out, hbicg_stats *fwd, hbicg_stats *adj);

/* One-call form with host pointers (creates and frees everything). */
int hbicg_solve(unsigned n, unsigned nnz, const unsigned *ptr, const unsigned *col, const double *val,
                const double *b, const double *sigma, int m, int seed, const hbicg_params *p, double *x,
                double *r_out, hbicg_stats *stats);

/* Solvers take their device buffers from a library-owned pool that keeps freed
 * memory for the next solver; this returns the memory no live solver uses to
 * the device (call it when the library's solves are done). */
void hbicg_release(void);

#ifdef __cplusplus
}
#endif
#endif /* HBICG_H */
