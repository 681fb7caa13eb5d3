/* TEST INFRASTRUCTURE — the oracle.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference legs may load this library, and only as
 * the checker or the timed CPU baseline, never as the product path.
 *
 * CPU restatement (plain C + OpenMP) of the reference's shifted BiCGStab with
 * seed switching, src/solver_dynamic.c:3-463 (variants src/solver_static.c,
 * src/solver_normal.c), and of its CSR SpMV, src/openmp_matrix.c:38-60.
 * Parity is pinned two ways: against the reference's own sources compiled
 * single-rank (oracle/_ref, see oracle/Makefile) and against the golden
 * vectors in tests/golden/ that the reference produced.
 */
#ifndef HBICG_ORACLE_H
#define HBICG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Schedules of the reference's three entry points (src/solver.h:33-35).  They
 * differ only in OpenMP scheduling, never in arithmetic. */
enum { HBO_SCHED_DYNAMIC = 0, HBO_SCHED_STATIC = 1, HBO_SCHED_NORMAL = 2 };

typedef struct {
    double tol;       /* relative tolerance, reference EPS (src/solver.h:13) */
    int max_iter;     /* reference MAX_ITER; the loop runs while k < max_iter+1 */
    int switching;    /* 1 = seed switching on (reference default, src/solver.h:31) */
    int schedule;     /* HBO_SCHED_* */
} hbo_opts;

typedef struct {
    /* switch log: at iteration sw_k[i] the seed became sw_seed[i] */
    int *sw_k, *sw_seed;
    int sw_cap, n_sw;
    /* act[k] = shifts updated by the shift loop at iteration k (1-based, k <= cap) */
    int *act;
    int act_cap;
    /* conv_k[j] = iteration at which shift j met the test (0 = never) */
    int *conv_k;
    int final_seed;
    /* optional per-iteration histories, index k = 1..(returned k - 1), capacity
     * hist_cap: the seed's alpha, beta, omega (as archived, i.e. rescaled after
     * a switch) and (r, r) at the end of iteration k */
    double *a_hist, *b_hist, *w_hist, *rr_hist;
    int hist_cap;
    /* optional wall-clock stamps (omp_get_wtime, seconds): t_iter[0] when the
     * iterations start (after the set-up), t_iter[k] at the end of iteration k */
    double *t_iter;
    int t_cap;
} hbo_trace;

/* y = A x for a square CSR matrix (32-bit indices): each row summed in stored
 * order, as src/openmp_matrix.c:44-58 does (y is overwritten). */
void hbo_spmv(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
              double *y);

/* y = A x with each row accumulated by fused multiply-adds in stored order. */
void hbo_spmv_fma(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
                  double *y);

/* Shifted BiCGStab with seed switching on (A + sigma_j I) x_j = b.
 * x: m*n doubles, shift-major, zero on entry.  r: b on entry, the final seed
 * residual on exit.  Returns k (iterations + 1 on convergence), exactly as the
 * reference does (src/solver_dynamic.c:461).  tr may be NULL. */
int hbo_shifted_bicgstab(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, double *x,
                         double *r, const double *sigma, int m, int seed, const hbo_opts *opt, hbo_trace *tr);

/* out[j] = ||b - (A + sigma_j I) x_j|| / ||b|| for every shift. */
void hbo_true_residuals(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
                        const double *b, const double *sigma, int m, double *out);

#ifdef __cplusplus
}
#endif
#endif
