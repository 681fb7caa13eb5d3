/* TEST INFRASTRUCTURE — the oracle (see hbicg_oracle.h for who may use it).
 *
 * CPU restatement of the reference's shifted BiCGStab with seed switching.
 * Every floating-point expression keeps the reference's operand order, so that
 * with contraction off (-ffp-contract=off, as oracle/Makefile builds it) the
 * results are bit-identical to the reference's own sources on any host:
 *   - seed BiCGStab step ................ src/solver_dynamic.c:156-210
 *   - shift recurrences and updates ..... src/solver_dynamic.c:239-256
 *   - convergence test + argmax ......... src/solver_dynamic.c:278-303
 *   - seed switch (rescale + replay) .... src/solver_dynamic.c:312-359
 * The parallel layout also follows the reference (one OpenMP region,
 * work-shared vector loops, dot products summed serially by the master thread
 * as my_openmp_ddot_v3 does, src/openmp_vector.c:60-76), so that the same code
 * serves as the timed CPU baseline where the reference itself cannot be built.
 */
#include "hbicg_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

/* ---- vector helpers (called inside an OpenMP parallel region) ------------ */

/* y[i] += a * x[i]  (src/openmp_vector.c:3-9) */
static void par_axpy(unsigned n, double a, const double *x, double *y) {
#pragma omp for
    for (long i = 0; i < (long)n; i++) y[i] += a * x[i];
}

static void par_scale(unsigned n, double a, double *x) {
#pragma omp for
    for (long i = 0; i < (long)n; i++) x[i] *= a;
}

static void par_copy(unsigned n, const double *x, double *y) {
#pragma omp for
    for (long i = 0; i < (long)n; i++) y[i] = x[i];
}

static void par_zero(unsigned n, double *x) {
#pragma omp for
    for (long i = 0; i < (long)n; i++) x[i] = 0.0;
}

/* Products in parallel, sum by the master in index order, then a barrier:
 * the result is independent of the thread count (src/openmp_vector.c:60-76). */
static void par_dot(unsigned n, const double *x, const double *y, double *tmp, double *out) {
#pragma omp for
    for (long i = 0; i < (long)n; i++) tmp[i] = x[i] * y[i];
#pragma omp master
    {
        double acc = 0.0;
        for (unsigned i = 0; i < n; i++) acc += tmp[i];
        *out = acc;
    }
#pragma omp barrier
}

/* y[i] += sum over the row in stored order; static or dynamic,1 schedule
 * (src/openmp_matrix.c:38-83). */
static void par_spmv_add(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
                         double *y, int dyn) {
    if (dyn) {
#pragma omp for schedule(dynamic, 1)
        for (long i = 0; i < (long)n; i++) {
            double acc = 0.0;
            for (unsigned e = ptr[i]; e < ptr[i + 1]; e++) acc += val[e] * x[col[e]];
            y[i] += acc;
        }
    } else {
#pragma omp for
        for (long i = 0; i < (long)n; i++) {
            double acc = 0.0;
            for (unsigned e = ptr[i]; e < ptr[i + 1]; e++) acc += val[e] * x[col[e]];
            y[i] += acc;
        }
    }
}

/* serial helpers used per shift and by the master (src/vector.c:3-21) */
static void ser_axpy(unsigned n, double a, const double *x, double *y) {
    for (unsigned i = 0; i < n; i++) y[i] += a * x[i];
}
static void ser_scale(unsigned n, double a, double *x) {
    for (unsigned i = 0; i < n; i++) x[i] *= a;
}
static double ser_dot(unsigned n, const double *x, const double *y) {
    double acc = 0.0;
    for (unsigned i = 0; i < n; i++) acc += x[i] * y[i];
    return acc;
}

void hbo_spmv(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
              double *y) {
#pragma omp parallel
    {
        par_zero(n, y);
        par_spmv_add(n, ptr, col, val, x, y, 0);
    }
}

/* The same row sums with every step a fused multiply-add (C99 fma, exact on
 * any host): acc = fma(val, x, acc) from acc = 0 in stored order.  This is
 * what a row loop compiled with contraction computes, and what the GPU SpMV
 * kernel computes per row. */
void hbo_spmv_fma(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
                  double *y) {
#pragma omp parallel for
    for (long i = 0; i < (long)n; i++) {
        double acc = 0.0;
        for (unsigned e = ptr[i]; e < ptr[i + 1]; e++) acc = fma(val[e], x[col[e]], acc);
        y[i] = acc;
    }
}

/* ---- the solver ----------------------------------------------------------- */

/* Per-shift scalar state.  pi holds the whole history pi_j[0..max_iter] of
 * every shift, shift-major, because a seed switch replays it from the start
 * (src/solver_dynamic.c:69,331-339). */
typedef struct {
    double *alpha, *beta, *omega, *eta, *zeta; /* per shift, the latest values */
    double *a_hist, *b_hist, *w_hist;          /* the seed's alpha/beta/omega per iteration */
    double *pi;                                /* [m][kcap] */
    unsigned char *done;
} shift_state;

int hbo_shifted_bicgstab(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, double *x,
                         double *r, const double *sigma, int m, int seed, const hbo_opts *opt, hbo_trace *tr) {
    const double tol = opt->tol;
    const int kcap = opt->max_iter + 1; /* loop bound and archive length */
    const int dyn_shift = (opt->schedule != HBO_SCHED_STATIC);
    const int dyn_spmv = 1; /* the second SpMV of every variant uses dynamic,1 */
    const int normal = (opt->schedule == HBO_SCHED_NORMAL);

    double *r_prev = malloc(sizeof(double) * n), *r_hat = malloc(sizeof(double) * n);
    double *s = malloc(sizeof(double) * n), *y = malloc(sizeof(double) * n);
    double *q_keep = malloc(sizeof(double) * n), *tmp = malloc(sizeof(double) * n);
    double *p = calloc((size_t)n * (size_t)m, sizeof(double));
    shift_state st;
    st.alpha = malloc(sizeof(double) * m);
    st.beta = malloc(sizeof(double) * m);
    st.omega = malloc(sizeof(double) * m);
    st.eta = malloc(sizeof(double) * m);
    st.zeta = malloc(sizeof(double) * m);
    st.a_hist = malloc(sizeof(double) * kcap);
    st.b_hist = malloc(sizeof(double) * kcap);
    st.w_hist = malloc(sizeof(double) * kcap);
    st.pi = malloc(sizeof(double) * (size_t)kcap * (size_t)m);
    st.done = calloc((size_t)m, 1);

    int k = 1, n_done = 0, argmax = seed;
    double rr_hat = ser_dot(n, r, r); /* (r^, r) with r^ = b */
    memcpy(r_hat, r, sizeof(double) * n);
    for (int j = 0; j < m; j++) {
        memcpy(p + (size_t)j * n, r, sizeof(double) * n);
        st.alpha[j] = 1.0;
        st.beta[j] = 0.0;
        st.eta[j] = 0.0;
        st.zeta[j] = 1.0;
        st.pi[(size_t)j * kcap + 0] = 1.0;
        if (kcap > 1) st.pi[(size_t)j * kcap + 1] = 1.0;
    }
    double rr = rr_hat, bb = rr_hat; /* (r, r) and (b, b) */
    double rs = 0.0, qq = 0.0, qy = 0.0, rr_hat_old = 0.0;
    st.a_hist[0] = 1.0;
    st.b_hist[0] = 0.0;
    if (tr) {
        tr->n_sw = 0;
        if (tr->conv_k) memset(tr->conv_k, 0, sizeof(int) * m);
        if (tr->t_iter && tr->t_cap > 0) tr->t_iter[0] = omp_get_wtime();
    }

#pragma omp parallel
    {
        while (n_done < m && k < kcap) {
            double *ps = p + (size_t)seed * n, *xs = x + (size_t)seed * n;
            const double sig_s = sigma[seed];

            /* seed step: s = (A + sigma_s I) p_s, alpha = (r^,r)/(r^,s) */
            par_copy(n, r, r_prev);
            par_zero(n, s);
            par_spmv_add(n, ptr, col, val, ps, s, normal);
            par_axpy(n, sig_s, ps, s);
            par_dot(n, r_hat, s, tmp, &rs);
#pragma omp master
            st.a_hist[k] = rr_hat / rs;
#pragma omp barrier
            const double ak = st.a_hist[k];

            /* q = r - alpha s (kept in r), y = (A + sigma_s I) q */
            par_axpy(n, -ak, s, r);
            par_copy(n, r, q_keep);
            par_zero(n, y);
            par_spmv_add(n, ptr, col, val, r, y, dyn_spmv);
            par_axpy(n, sig_s, r, y);
            par_dot(n, r, r, tmp, &qq);
            par_dot(n, r, y, tmp, &qy);
#pragma omp master
            {
                st.w_hist[k] = qq / qy;
                rr_hat_old = rr_hat;
            }
#pragma omp barrier
            const double wk = st.w_hist[k];

            /* x_s += alpha p_s + omega q ; r = q - omega y */
            par_axpy(n, ak, ps, xs);
            par_axpy(n, wk, r, xs);
            par_axpy(n, -wk, y, r);
            par_dot(n, r, r, tmp, &rr);
            par_dot(n, r_hat, r, tmp, &rr_hat);
#pragma omp master
            st.b_hist[k] = (st.a_hist[k] / st.w_hist[k]) * (rr_hat / rr_hat_old);
#pragma omp barrier
            const double bk = st.b_hist[k];

            /* p_s = beta p_s + r - beta omega s */
            par_scale(n, bk, ps);
            par_axpy(n, 1.0, r, ps);
            par_axpy(n, -bk * wk, s, ps);

            /* every unconverged shift from the seed's scalars */
            const double ratio_prev = st.b_hist[k - 1] / st.a_hist[k - 1];
            if (dyn_shift) {
#pragma omp for schedule(dynamic, 1)
                for (int j = 0; j < m; j++) {
                    if (j == seed || st.done[j]) continue;
                    double *pij = st.pi + (size_t)j * kcap;
                    double *xj = x + (size_t)j * n, *pj = p + (size_t)j * n;
                    const double d = sig_s - sigma[j];
                    st.eta[j] = ratio_prev * ak * st.eta[j] - d * ak * pij[k - 1];
                    pij[k] = st.eta[j] + pij[k - 1];
                    st.alpha[j] = (pij[k - 1] / pij[k]) * ak;
                    st.omega[j] = wk / (1.0 - wk * d);
                    ser_axpy(n, st.omega[j] / (pij[k] * st.zeta[j]), q_keep, xj);
                    ser_axpy(n, st.alpha[j], pj, xj);
                    ser_axpy(n, st.omega[j] / (st.alpha[j] * st.zeta[j] * pij[k]), q_keep, pj);
                    ser_axpy(n, -st.omega[j] / (st.alpha[j] * st.zeta[j] * pij[k - 1]), r_prev, pj);
                    st.zeta[j] = (1.0 - wk * d) * st.zeta[j];
                    st.beta[j] = (pij[k - 1] / pij[k]) * (pij[k - 1] / pij[k]) * bk;
                    ser_scale(n, st.beta[j], pj);
                    ser_axpy(n, 1.0 / (pij[k] * st.zeta[j]), r, pj);
                }
            } else {
#pragma omp for
                for (int j = 0; j < m; j++) {
                    if (j == seed || st.done[j]) continue;
                    double *pij = st.pi + (size_t)j * kcap;
                    double *xj = x + (size_t)j * n, *pj = p + (size_t)j * n;
                    const double d = sig_s - sigma[j];
                    st.eta[j] = ratio_prev * ak * st.eta[j] - d * ak * pij[k - 1];
                    pij[k] = st.eta[j] + pij[k - 1];
                    st.alpha[j] = (pij[k - 1] / pij[k]) * ak;
                    st.omega[j] = wk / (1.0 - wk * d);
                    ser_axpy(n, st.omega[j] / (pij[k] * st.zeta[j]), q_keep, xj);
                    ser_axpy(n, st.alpha[j], pj, xj);
                    ser_axpy(n, st.omega[j] / (st.alpha[j] * st.zeta[j] * pij[k]), q_keep, pj);
                    ser_axpy(n, -st.omega[j] / (st.alpha[j] * st.zeta[j] * pij[k - 1]), r_prev, pj);
                    st.zeta[j] = (1.0 - wk * d) * st.zeta[j];
                    st.beta[j] = (pij[k - 1] / pij[k]) * (pij[k - 1] / pij[k]) * bk;
                    ser_scale(n, st.beta[j], pj);
                    ser_axpy(n, 1.0 / (pij[k] * st.zeta[j]), r, pj);
                }
            }

#pragma omp master
            {
                /* convergence test on the recursive residual; strict '>' argmax
                 * starting from 1.0 keeps the lowest index on exact ties */
                int active = 0;
                double best = 1.0;
                for (int j = 0; j < m; j++) {
                    if (st.done[j]) continue;
                    if (j != seed) active++;
                    double a = (j == seed) ? 1.0 : fabs(1.0 / (st.zeta[j] * st.pi[(size_t)j * kcap + k]));
                    if (a * a * rr <= tol * tol * bb) {
                        st.done[j] = 1;
                        n_done++;
                        if (tr && tr->conv_k) tr->conv_k[j] = k;
                    } else if (a > best) {
                        best = a;
                        argmax = j;
                    }
                }
                if (tr && tr->act && k < tr->act_cap) tr->act[k] = active;
                if (tr && tr->rr_hist && k < tr->hist_cap) tr->rr_hist[k] = rr;

                if (opt->switching && st.done[seed] && n_done < m) {
                    const int t = argmax;
                    const double *pit = st.pi + (size_t)t * kcap;
                    const double dst = sigma[seed] - sigma[t];
                    for (int i = 1; i <= k; i++) {
                        st.a_hist[i] = (pit[i - 1] / pit[i]) * st.a_hist[i];
                        st.b_hist[i] = (pit[i - 1] / pit[i]) * (pit[i - 1] / pit[i]) * st.b_hist[i];
                        st.w_hist[i] = st.w_hist[i] / (1.0 - st.w_hist[i] * dst);
                    }
                    ser_scale(n, 1.0 / (st.zeta[t] * pit[k]), r);
                    rr_hat = ser_dot(n, r_hat, r);
                    for (int j = 0; j < m; j++) {
                        st.eta[j] = 0.0;
                        st.zeta[j] = 1.0;
                    }
                    for (int i = 1; i <= k; i++) {
                        for (int j = 0; j < m; j++) {
                            if (st.done[j] || j == t) continue;
                            double *pij = st.pi + (size_t)j * kcap;
                            const double d = sigma[t] - sigma[j];
                            st.eta[j] = (st.b_hist[i - 1] / st.a_hist[i - 1]) * st.a_hist[i] * st.eta[j] -
                                        d * st.a_hist[i] * pij[i - 1];
                            pij[i] = st.eta[j] + pij[i - 1];
                            st.zeta[j] = (1.0 - st.w_hist[i] * d) * st.zeta[j];
                        }
                    }
                    seed = t;
                    if (tr && tr->n_sw < tr->sw_cap) {
                        tr->sw_k[tr->n_sw] = k;
                        tr->sw_seed[tr->n_sw] = t;
                    }
                    if (tr) tr->n_sw++;
                }
                if (tr && tr->t_iter && k < tr->t_cap) tr->t_iter[k] = omp_get_wtime();
                k++;
            }
#pragma omp barrier
        }
    }

    if (tr) {
        tr->final_seed = seed;
        for (int i = 0; i < k && i < tr->hist_cap; i++) {
            if (tr->a_hist) tr->a_hist[i] = st.a_hist[i];
            if (tr->b_hist) tr->b_hist[i] = st.b_hist[i];
            if (tr->w_hist) tr->w_hist[i] = i ? st.w_hist[i] : 0.0;
        }
    }
    free(r_prev); free(r_hat); free(s); free(y); free(q_keep); free(tmp); free(p);
    free(st.alpha); free(st.beta); free(st.omega); free(st.eta); free(st.zeta);
    free(st.a_hist); free(st.b_hist); free(st.w_hist); free(st.pi); free(st.done);
    return k;
}

void hbo_true_residuals(unsigned n, const unsigned *ptr, const unsigned *col, const double *val, const double *x,
                        const double *b, const double *sigma, int m, double *out) {
    double bnorm2 = 0.0;
    for (unsigned i = 0; i < n; i++) bnorm2 += b[i] * b[i];
    for (int j = 0; j < m; j++) {
        const double *xj = x + (size_t)j * n;
        double acc = 0.0;
#pragma omp parallel for reduction(+ : acc)
        for (long i = 0; i < (long)n; i++) {
            double ax = 0.0;
            for (unsigned e = ptr[i]; e < ptr[i + 1]; e++) ax += val[e] * xj[col[e]];
            double res = b[i] - (ax + sigma[j] * xj[i]);
            acc += res * res;
        }
        out[j] = sqrt(acc) / sqrt(bnorm2);
    }
}
