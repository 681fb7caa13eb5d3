/* Thin C ABI between the C host code (solver driver, loaders) and the sm_103a
 * CUDA kernels of the shifted BiCGStab solver.  Everything here is plain C:
 * device pointers, sizes and a stream.  The structs describe how the solver
 * lays its data out in HBM:
 *   - the matrix: CSR with 32-bit row pointers and column indices and FP64
 *     values, plus the SpMV schedule (row blocks) built once per matrix;
 *   - per-shift vectors x_j, p_j: shift-major [m][n] FP64 arrays;
 *   - the Krylov basis (deferred mode): slots of n doubles, [L][n];
 *   - the scalar state of the iteration (seed scalars, per-shift recurrences,
 *     the alpha/beta/omega history and the pi archive), all device-resident so
 *     that a whole iteration runs without a host round trip.
 */
#ifndef HBK_H
#define HBK_H

#include <cuda_runtime.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HBK_THREADS 256      /* threads per block of every streaming kernel */
#define HBK_MAX_GRID 4096    /* upper bound on persistent grids (partial-sum slots) */
#define HBK_TILE_NNZ 2048    /* nonzeros staged in shared memory per SpMV row block */
#define HBK_NCOEF 8          /* coefficients per shift per iteration */

/* status bits (device and host) */
#define HBK_ST_BREAKDOWN 1   /* a scalar of the recurrence became 0, inf or nan */
#define HBK_ST_BASIS_FULL 2  /* deferred mode: the basis needs a flush */
#define HBK_ST_SHIFT_FAIL 4  /* a non-seed shift broke down (its conv_k is -k) and stopped */

/* SpMV row-block kinds (bits 30..31 of blk_row entries are not used; kinds
 * are a separate byte array) */
#define HBK_BLK_TILE 0       /* up to HBK_THREADS short rows, <= HBK_TILE_NNZ nonzeros */
#define HBK_BLK_LONG 1       /* one long row, reduced by the whole block */

/* SpMV storage formats */
#define HBK_FMT_TILE 0       /* CSR, row blocks staged in shared memory */
#define HBK_FMT_SELL 1       /* SELL-32: slices of 32 rows, column-major within a slice */
#define HBK_SELL_MAX_LEN 64  /* longest row the SELL format takes */
#define HBK_FMT_HYB 2        /* short rows in SELL-32 slices (length-sorted inside windows), long rows one warp each */
#define HBK_HYB_SHORT 32     /* longest row of a HYB slice */
#define HBK_HYB_WINDOW 1024  /* rows are sorted by length only inside windows of this many consecutive rows */
#define HBK_HYB_L4 128       /* long rows up to this length: 4 lanes each, 8 rows per warp */
#define HBK_HYB_L16 512      /* longer rows up to this length: 16 lanes each, 2 rows per warp; longer: a warp */
#define HBK_FMT_MERGE 3      /* CSR; rows up to HBK_MERGE_LONG entries in merge-path blocks, longer rows one warp each */
#define HBK_MERGE_IPT 8      /* merge items (row ends + nonzeros) per lane of a block */
#define HBK_MERGE_ITEMS (32 * HBK_MERGE_IPT) /* items per block (one warp) */
#define HBK_MERGE_LONG (HBK_MERGE_ITEMS - 1) /* longest row a merge block takes (the row and its end fill it) */

typedef struct {
    unsigned n, nnz;
    const unsigned *ptr, *col; /* device CSR, n+1 and nnz entries */
    const double *val;
    const unsigned *blk_row;   /* device: first row of each row block, nblk+1 entries */
    const unsigned char *blk_kind;
    unsigned nblk;
    int grid;                  /* persistent grid of the SpMV kernels */
    int fmt;                   /* HBK_FMT_* */
    const double *sval;        /* SELL: values, slice s at sptr[s], entry e of lane l at +e*32+l */
    const unsigned *scol;      /* SELL: column indices (padding: the row itself, value 0) */
    const unsigned long long *sptr; /* SELL: n/32 rounded up + 1 slice offsets; HYB: nslice + 1 */
    unsigned long long sell_len;    /* SELL: entries of sval/scol (with padding) */
    const unsigned *srow;      /* HYB: row of slice s, lane l at 32 s + l (>= n: an empty lane) */
    const unsigned char *slen; /* HYB: length of that row (0: an empty lane) */
    unsigned nslice;           /* HYB: slices of short rows */
    const unsigned *wrow;      /* HYB: rows longer than HBK_HYB_SHORT, longest first, one warp each */
    unsigned nwrow;
    const unsigned *wrng;      /* HYB: first and end entry of long row i at 2 i, 2 i + 1 */
    const unsigned *hwbeg;     /* HYB: work list of warp w = items hitem[hwbeg[w] .. hwbeg[w + 1]) */
    const unsigned *hitem;     /* HYB: work items (hbk_hyb_classes), then slice i - hitl */
    unsigned hnw;              /* HYB: warps the lists were balanced for */
    unsigned hrow32, hrow16;   /* HYB: long rows [0, hrow32) have 32 lanes each, [hrow32, hrow16) 16, the rest 4 */
    unsigned hit16, hit4, hitl; /* HYB: first item of 16-lane rows, of 4-lane rows, of the slices */
    const unsigned *mblk;      /* MERGE: [2 nmblk] first and end row of each block of short rows */
    unsigned nmblk;
    const unsigned *mlong;     /* MERGE: rows longer than HBK_MERGE_LONG, longest first, one warp each */
    unsigned nmlong;
} hbk_matrix;

/* Device-resident scalars of one solve. */
typedef struct {
    double rr_hat;      /* (r^, r) */
    double rr_hat_old;
    double rr;          /* (r, r) at the end of the current iteration */
    double bb;          /* (b, b) */
    double rs, qq, qy;  /* raw reductions of the current iteration */
    double alpha, omega, beta;
    double r_scale;     /* 1 / (zeta_t pi_t) when the iteration ends with a switch */
    double tol;
    int k;              /* current iteration, 1-based */
    int seed;           /* seed of the current iteration */
    int next_seed;
    int n_done;         /* converged systems */
    int finished;       /* set once n_done == m or k == kcap */
    int switched;       /* this iteration ends with a seed switch */
    int n_active;       /* entries in act_list for the shift update */
    int status;         /* HBK_ST_* */
    int n_sw;           /* seed switches so far */
    int max_sigma;      /* the argmax of the last convergence test */
    int m, kcap;        /* shifts, history length (max_iter + 1) */
    int switching;      /* 1 = seed switching on */
    int slots;          /* deferred mode: basis slots in use */
    int slot_r_old;     /* deferred mode: slot of r_{k-1} */
    int slot_cap;
    int need_ps;        /* deferred mode: the new seed's p must be formed from the basis */
    double rs_switch;   /* (r^, r_k) after the switch rescale */
    int loops;          /* bodies of the device-side iteration loop run in this solve (bound on the loop) */
} hbk_scalars;

typedef struct {
    hbk_scalars *sc;
    const double *sigma;        /* [m] */
    double *a_hist, *b_hist, *w_hist; /* [kcap] seed alpha / beta / omega history */
    double *pi;                 /* [m][kcap] */
    double *eta, *zeta;         /* [m] */
    int *done, *conv_k;         /* [m]; conv_k: iteration of convergence, -k for a shift that broke down at k */
    int *act_list;              /* [m] shifts updated this iteration */
    double *coef;               /* [m][HBK_NCOEF] their coefficients */
    int *sw_k, *sw_seed;        /* [m] switch log */
    int *act_hist;              /* [kcap] active non-seed shifts per iteration */
    double *partials;           /* [4][HBK_MAX_GRID] */
    unsigned *counters;         /* [8] last-block tickets */
    double *ratio;              /* [kcap] scratch for the switch replay */
    int *lslot;                 /* [m] deferred mode: basis slots in use at a system's last update */
    double *rr_hist;            /* [kcap] (r, r) at the end of each iteration */
    int m, kcap;
} hbk_shifts;

/* Deferred mode keeps x_j and the flushed p_j panel-major: element i of
 * system j at ((i / HBK_PANEL) m + j) HBK_PANEL + i % HBK_PANEL.  The basis
 * flush forms every system's values for one panel of HBK_PANEL elements at a
 * time, so it reads and writes one contiguous block per panel instead of m
 * rows that lie n elements apart. */
#define HBK_PANEL 48
/* entries per basis slot of the slot-maximum array (spreads the atomics) */
#define HBK_SLOT_SPREAD 32
static inline size_t hbk_panel_elems(unsigned n, int m) {
    return ((size_t)n + HBK_PANEL - 1) / HBK_PANEL * HBK_PANEL * (size_t)(m > 0 ? m : 1);
}

typedef struct {
    unsigned n;
    double *r_hat;              /* shadow residual = b */
    double *rbuf[2];            /* r_{k-1} / r_k, alternating with k */
    double *s, *q, *y;
    double *X, *P;              /* [m][n] shift-major (P unused in deferred mode; X written at the end) */
    /* deferred (Krylov basis) mode */
    double *V;                  /* [slot_cap][n] */
    double *ps;                 /* the seed's search vector */
    double *Xc, *Pc;            /* [m][slot_cap] coefficients */
    double *own;                /* [m][2]: coefficient of the flushed p_j in x_j and in p_j */
    double *Pmat;               /* flushed p_j, panel-major (allocated on the first flush) */
    double *Xp;                 /* x_j during the solve, panel-major */
    unsigned long long *slot_max; /* [slot_cap][HBK_SLOT_SPREAD] bits of max |V[l]|: the kernels that write a
                                     slot fold block b's maximum into entry b % HBK_SLOT_SPREAD */
    /* seed shift folded into the SELL-32 diagonal (deferred mode): the seed
     * kernels' products read sval_shift = sval with sigma_seed added at each
     * row's diagonal entry (position sdiag[row]) instead of adding sigma x */
    double *sval_shift;
    const double *sval_orig;
    const unsigned long long *sdiag;
    int pm;                     /* systems per panel (m) */
    int slot_cap;
    int deferred;
} hbk_vectors;

/* ---- plain BLAS-1 and SpMV kernels (one launch per reference step) ---- */
int hbk_copy(unsigned n, const double *x, double *y, cudaStream_t st);
int hbk_zero(unsigned n, double *x, cudaStream_t st);
int hbk_axpy(unsigned n, double a, const double *x, double *y, cudaStream_t st);
int hbk_scal(unsigned n, double a, double *x, cudaStream_t st);
int hbk_fill(unsigned n, double v, double *x, cudaStream_t st);
/* deterministic dot: result written to *out (device), fixed summation tree */
int hbk_dot(unsigned n, const double *x, const double *y, double *partials, unsigned *counter, double *out,
            cudaStream_t st);
/* the same on at most grid_cap blocks (partials holds grid_cap doubles) */
int hbk_dot_capped(unsigned n, const double *x, const double *y, int grid_cap, double *partials, unsigned *counter,
                   double *out, cudaStream_t st);
/* y = A x (+ sigma * x when sigma_add != 0), rows summed in stored order by one thread */
int hbk_spmv(const hbk_matrix *A, const double *x, double *y, double sigma, int sigma_add, cudaStream_t st);
/* y += A x (the reference's mult accumulates into y) */
int hbk_spmv_accumulate(const hbk_matrix *A, const double *x, double *y, cudaStream_t st);

/* ---- SpMV schedule ---- */
/* Host: split rows into blocks (counts only when blk_row is NULL). */
unsigned hbk_plan_rows(unsigned n, const unsigned *ptr_host, unsigned *blk_row, unsigned char *blk_kind);
int hbk_spmv_grid(unsigned nblk);
/* MERGE form: CTAs of one wave of the product kernel, at most `units` */
int hbk_merge_grid(unsigned units);
/* SELL-32 build on the device: widths of the ceil(n/32) slices into w ... */
int hbk_sell_widths(unsigned n, const unsigned *ptr, unsigned *w, cudaStream_t st);
/* ... then, with sptr = exclusive prefix sum of 32*w (host), fill the arrays */
/* one-wave grid (blocks) of the kernels that take the HYB form */
int hbk_hyb_wave_fused(void);
int hbk_hyb_wave_blas(void);
/* HYB slices: slice s, lane l holds row srow[32 s + l] (entry e at sptr[s] + 32 e + l) */
int hbk_hyb_fill(unsigned nslice, const unsigned *srow, unsigned n, const unsigned *ptr, const unsigned *col,
                 const double *val, const unsigned long long *sptr, double *sval, unsigned *scol, cudaStream_t st);
/* sdiag[r] = position in the SELL-32 arrays of row r's first stored diagonal
 * entry; *missing = 1 when some row has none */
int hbk_sell_diag(unsigned n, const unsigned *ptr, const unsigned long long *sptr, const unsigned *scol,
                  unsigned long long *sdiag, int *missing, cudaStream_t st);
/* sval_shift = sval (len entries) with *sigma (device) added at every row's diagonal */
int hbk_fold_diag(unsigned n, const double *sval, unsigned long long len, const unsigned long long *sdiag,
                  const double *sigma, double *sval_shift, cudaStream_t st);
int hbk_sell_fill(unsigned n, const unsigned *ptr, const unsigned *col, const double *val,
                  const unsigned long long *sptr, double *sval, unsigned *scol, cudaStream_t st);

/* ---- fused solver ---- */
int hbk_fused_init(const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, const double *b, int seed,
                   double tol, cudaStream_t st);
int hbk_fused_iteration(const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, cudaStream_t st);
/* end of one body of a CUDA graph's conditional while loop over iterations:
 * sets the loop's condition to "not finished", and to 0 once the solve has run
 * loop_cap bodies (a bound on the loop whatever the scalars say) */
int hbk_loop_condition(const hbk_shifts *sh, cudaGraphConditionalHandle cond, int loop_cap, cudaStream_t st);
/* Many families' iterations in one persistent cooperative launch: every
 * family in the fused form on SELL-32, either shift mode, already set up by
 * hbk_fused_init; the launch runs until every family has stopped or paused
 * with a full basis (or iter_cap iterations).  A[f], v[f], sh[f] describe
 * family f; rows_per_vb: rows of a family per virtual block (0:
 * HBK_GROUP_ROWS); ws: device memory of hbk_group_ws_bytes(nf, v,
 * rows_per_vb) bytes; max_ctas > 0 caps the CTAs (else one wave,
 * hbk_group_ctas(0); never more than the virtual blocks).  Returns after the
 * launch has ended; *err_out: 0, HBK_GROUP_ERR_WAIT (a grid barrier's wait
 * ran out) or HBK_GROUP_ERR_CAP (iter_cap reached with a family still
 * running). */
#define HBK_GROUP_ROWS 1024              /* default rows of a family per virtual block */
#define HBK_GROUP_WAIT_NS 2000000000ull  /* longest wait at a grid barrier */
#define HBK_GROUP_ERR_WAIT 1
#define HBK_GROUP_ERR_CAP 2
size_t hbk_group_ws_bytes(int nf, const hbk_vectors *v, unsigned rows_per_vb);
int hbk_group_ctas(int max_ctas);
int hbk_group_run(int nf, const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, int iter_cap, int max_ctas,
                  unsigned rows_per_vb, void *ws, size_t ws_bytes, int *err_out, cudaStream_t st);
/* test of the bounded barrier wait: the next hbk_group_run's CTA 0 does not
 * arrive at its first barrier, so every CTA waits out HBK_GROUP_WAIT_NS and
 * the launch ends with HBK_GROUP_ERR_WAIT (one shot) */
void hbk_group_test_withhold(int on);
/* deferred mode: x_j (and p_j when keep_p) = coefficients x basis, then reset the basis */
int hbk_deferred_flush(const hbk_vectors *v, const hbk_shifts *sh, int keep_p, cudaStream_t st);
/* ||b - (A + sigma_j I) x_j||^2 for every shift into out[m] (device) */
int hbk_true_residuals(const hbk_matrix *A, const double *X, const double *b, const double *sigma, int m,
                       double *partials, unsigned *counter, double *out, cudaStream_t st);

/* basis flush on the tensor cores (flush_tc.cu): x_j += xi_j Pmat_j + Xc_j . V,
 * p_j = rho_j Pmat_j + Pc_j . V over the first L <= hbk_flush_tc_max_slots()
 * slots, FP64-accurate; X and Pmat panel-major (HBK_PANEL) with m systems;
 * ws of hbk_flush_tc_workspace_bytes(m) bytes; *err set on a bounded-wait
 * timeout.  No reset (see hbk_deferred_reset). */
/* COO -> CSR on the device, stable within rows (csrc/coo_csr.cu) */
size_t hbk_coo_to_csr_tmp_bytes(unsigned nnz);
int hbk_coo_to_csr(unsigned n, unsigned nnz, const unsigned *row, const unsigned *col, const double *val,
                   unsigned *ptr, unsigned *col_out, double *val_out, void *tmp, int *err, cudaStream_t st);
/* adjoint gradients (csrc/adjoint.cu) */
int hbk_entry_rows(unsigned n, const unsigned *ptr, unsigned *rows, cudaStream_t st);
size_t hbk_adjoint_tmp_bytes(int m);
int hbk_shift_dots(unsigned n, int m, const double *X, size_t ldx, const double *a, size_t lda, int a_shared,
                   const double *w, double scale, double *out, void *tmp, cudaStream_t st);
int hbk_grad_b(unsigned n, int m, const double *Y, size_t ldy, const double *w, double *db, cudaStream_t st);
int hbk_grad_val(unsigned nnz, const unsigned *rows, const unsigned *col, int m, const double *X, size_t ldx,
                 const double *Y, size_t ldy, const double *w, double *dval, cudaStream_t st);
size_t hbk_flush_tc_workspace_bytes(int m);
int hbk_flush_tc_max_slots(void);
int hbk_flush_tc_run(const double *V, size_t ld, unsigned n, int L, const double *Xc, const double *Pc, int cap,
                     const double *own, int m, double *X, double *Pmat, int keep_p, void *ws, int *err,
                     cudaStream_t st);
/* the same for the live shifts only (conv_k[j] == 0 or conv_k[j] > k_last; the
 * others' rows are left as they are); conv_k: device [m] or NULL (all live);
 * slot_max: device [L][HBK_SLOT_SPREAD] partial maxima of each slot's |value|
 * (bits), or NULL (computed) */
int hbk_flush_tc_run_live(const double *V, size_t ld, unsigned n, int L, const double *Xc, const double *Pc, int cap,
                          const double *own, int m, double *X, double *Pmat, int keep_p, const int *conv_k,
                          int k_last, const unsigned long long *slot_max, void *ws, int *err, cudaStream_t st);
const int *hbk_flush_tc_live_count(const void *ws, int m); /* device int: live shifts of the last run on ws */
/* x[i] = element i of system j of the panel-major Xp (m systems), i < n */
int hbk_panel_row(const double *Xp, int m, unsigned n, int j, double *x, cudaStream_t st);
/* X[j][i] (leading dimension ld) = Xp in panel layout with m systems, i < n */
int hbk_panel_to_rows(const double *Xp, int m, unsigned n, double *X, size_t ld, cudaStream_t st);
/* after a flush: zero the coefficients, own = (0, keep_p), basis slot 0 = r_{k-1} */
int hbk_deferred_reset(const hbk_vectors *v, const hbk_shifts *sh, int keep_p, cudaStream_t st);

/* the same with an explicit leading dimension of X and at most grid_cap blocks */
int hbk_true_residuals_ld(const hbk_matrix *A, const double *X, size_t ldx, const double *b, const double *sigma,
                          int m, int grid_cap, double *partials, unsigned *counters, double *out, cudaStream_t st);

int hbk_last_error(void);
const char *hbk_error_string(int code);
int hbk_device_sm_count(void);

#ifdef __cplusplus
}
#endif
#endif
