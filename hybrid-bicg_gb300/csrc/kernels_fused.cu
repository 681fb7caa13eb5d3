// Fused shifted BiCGStab iteration with on-device scalars and seed switching.
//
// One iteration is five launches (seven in deferred mode), each reading the
// device-resident scalars, so an iteration (or a CUDA graph of many) needs no
// host round trip:
//   K1 seed_s     s = (A + sigma_s I) p_s, (r^,s) fused        -> alpha
//   K2 seed_q     q = r_{k-1} - alpha s
//   K3 seed_y     y = (A + sigma_s I) q, (q,q), (q,y) fused     -> omega
//   K4 seed_upd   x_s += alpha p_s + omega q ; r_k = q - omega y ; (r,r), (r^,r)
//                 last block: beta, every shift's recurrence and coefficients,
//                 the convergence test, argmax and the seed switch
//   K5 shifts     p_s and every unconverged shift's x_j, p_j in one pass
//                 (incremental mode); r_k rescaled on a switch
//   K6/K7         deferred mode only: coefficient update of every system in
//                 the Krylov basis; materialise the new seed's p after a switch
// Reference: src/solver_dynamic.c:147-381 (seed step :156-210, shift loop
// :239-256, convergence test :278-303, seed switch :312-359).
#include <vector>

#include "hbk_device.cuh"


using namespace hbk;

namespace {

// Scalar arithmetic of the recurrences is written with explicit round-to-nearest
// operations so no multiply-add is contracted: the recurrences then round
// exactly as the reference's C does for the same inputs.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

struct Ctx {
    hbk_matrix A;
    hbk_vectors v;
    hbk_shifts sh;
};

__device__ __forceinline__ size_t ldn(unsigned n) { return ((size_t)n + 31) / 32 * 32; }

__device__ __forceinline__ const double *seed_p(const Ctx &c, int seed) {
    return c.v.deferred ? c.v.ps : c.v.P + (size_t)seed * ldn(c.v.n);
}
__device__ __forceinline__ double *vec_r_old(const Ctx &c, const hbk_scalars *sc) {
    return c.v.deferred ? c.v.V + (size_t)sc->slot_r_old * ldn(c.v.n) : c.v.rbuf[(sc->k - 1) & 1];
}
__device__ __forceinline__ double *vec_r_new(const Ctx &c, const hbk_scalars *sc) {
    return c.v.deferred ? c.v.V + (size_t)(sc->slots + 1) * ldn(c.v.n) : c.v.rbuf[sc->k & 1];
}
__device__ __forceinline__ double *vec_q(const Ctx &c, const hbk_scalars *sc) {
    return c.v.deferred ? c.v.V + (size_t)sc->slots * ldn(c.v.n) : c.v.q;
}

// (an L2 load: in a persistent launch another CTA may have set the flag
// since this SM last read it)
__device__ __forceinline__ bool stopped(const hbk_scalars *sc) { return __ldcg(&sc->finished) != 0; }

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_init(Ctx c, int seed, double tol) {
    hbk_scalars *sc = c.sh.sc;
    const int m = c.sh.m, kcap = c.sh.kcap;
    for (int j = threadIdx.x; j < m; j += NT) {
        double *pij = c.sh.pi + (size_t)j * kcap;
        pij[0] = 1.0;
        if (kcap > 1) pij[1] = 1.0;
        c.sh.eta[j] = 0.0;
        c.sh.zeta[j] = 1.0;
        c.sh.done[j] = 0;
        c.sh.conv_k[j] = 0;
    }
    for (int i = threadIdx.x; i < 8; i += NT) c.sh.counters[i] = 0;
    if (threadIdx.x == 0) {
        c.sh.a_hist[0] = 1.0;
        c.sh.b_hist[0] = 0.0;
        c.sh.w_hist[0] = 0.0;
        const double bb = sc->bb;  // written by the (b,b) reduction launched just before
        sc->rr_hat = bb;
        sc->rr_hat_old = bb;
        sc->rr = bb;
        sc->alpha = sc->omega = sc->beta = 0.0;
        sc->r_scale = 1.0;
        sc->tol = tol;
        sc->k = 1;
        sc->seed = seed;
        sc->next_seed = seed;
        sc->n_done = 0;
        sc->switched = 0;
        sc->n_active = 0;
        sc->status = 0;
        sc->n_sw = 0;
        sc->loops = 0;
        sc->max_sigma = seed;
        sc->m = m;
        sc->kcap = kcap;
        sc->slots = 1;
        sc->slot_r_old = 0;
        sc->slot_cap = c.v.slot_cap;
        sc->need_ps = 0;
        sc->finished = (m <= 0 || kcap <= 1) ? 1 : 0;
        if (bb == 0.0) {  // b = 0: x = 0 solves every system exactly
            sc->finished = 1;
            sc->n_done = m;
        }
    }
}

// deferred mode: X = 0, Xc = 0, Pc[j][0] = 1 (p_j = b = basis slot 0), own = (0, 0)
__global__ void __launch_bounds__(NT) k_init_coef(Ctx c) {
    const int m = c.sh.m, cap = c.v.slot_cap;
    const size_t tot = (size_t)m * cap;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < tot; i += (size_t)gridDim.x * NT) {
        c.v.Xc[i] = 0.0;
        c.v.Pc[i] = (i % cap == 0) ? 1.0 : 0.0;
    }
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < (size_t)m; i += (size_t)gridDim.x * NT) {
        c.v.own[2 * i] = 0.0;
        c.v.own[2 * i + 1] = 0.0;
        c.sh.lslot[i] = 1;
    }
}

// ---------------------------------------------------------------------------
// K1: s = (A + sigma_s I) p_s and (r^, s)
template <int FMT, class G>
__device__ __forceinline__ void seed_s_body(const Ctx &c, const G &g) {
    __shared__ double red[2 * NW];
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const int seed = sc->seed;
    const double sig = c.sh.sigma[seed];
    const double *__restrict__ ps = seed_p(c, seed);
    const double *__restrict__ rh = c.v.r_hat;
    double *__restrict__ s = c.v.s;
    const bool folded = c.v.sval_shift != nullptr;  // the product already holds sigma p
    double acc = 0.0;
    auto epi = [&](unsigned r, double ax) {
        const double sv = folded ? ax : fma(sig, HBK_LD(G, ps, r), ax);
        s[r] = sv;
        acc = fma(HBK_LD(G, rh, r), sv, acc);
    };
    spmv_rows<FMT>(c.A, ps, epi, g);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) c.sh.partials[g.b()] = acc;
    if (take_ticket(c.sh.counters + 0, g.nb())) {
        const double rs = sum_partials(c.sh.partials, g.nb(), red);
        if (threadIdx.x == 0) {
            const int k = sc->k;
            const double a = dvd(sc->rr_hat, rs);
            sc->rs = rs;
            c.sh.a_hist[k] = a;
            sc->alpha = a;
            if (!fin(a)) {
                sc->status |= HBK_ST_BREAKDOWN;
                sc->finished = 1;
            }
            c.sh.counters[0] = 0;
        }
    }
}
template <int FMT>
__global__ void __launch_bounds__(NT) k_seed_s(Ctx c) { seed_s_body<FMT>(c, HwGrid()); }
template <>
__global__ void __launch_bounds__(NT, HBK_HYB_MINB) k_seed_s<HBK_FMT_HYB>(Ctx c) {
    seed_s_body<HBK_FMT_HYB>(c, HwGrid());
}

// K2: q = r_{k-1} - alpha s (deferred mode: q is a basis slot; its max |q| is
// kept for the flush)
template <class G>
__device__ __forceinline__ void seed_q_body(const Ctx &c, const G &g) {
    __shared__ unsigned long long smx[NW];
    const hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const double a = sc->alpha;
    const double *__restrict__ ro = vec_r_old(c, sc);
    const double *__restrict__ s = c.v.s;
    double *__restrict__ q = vec_q(c, sc);
    const unsigned n = c.v.n;
    unsigned long long mx = 0;
    for (size_t i = g.b() * (size_t)NT + threadIdx.x; i < n; i += (size_t)g.nb() * NT) {
        const double qi = fma(-a, HBK_LD(G, s, i), HBK_LD(G, ro, i));
        q[i] = qi;
        const unsigned long long b = abs_bits(qi);
        mx = b > mx ? b : mx;
    }
    if (c.v.slot_max) block_max_to(mx, smx, c.v.slot_max + (size_t)sc->slots * HBK_SLOT_SPREAD);
}
__global__ void __launch_bounds__(NT) k_seed_q(Ctx c) { seed_q_body(c, HwGrid()); }

// K3: y = (A + sigma_s I) q, (q,q) and (q,y)
template <int FMT, class G>
__device__ __forceinline__ void seed_y_body(const Ctx &c, const G &g) {
    __shared__ double red[2 * NW];
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const double sig = c.sh.sigma[sc->seed];
    const double *__restrict__ q = vec_q(c, sc);
    double *__restrict__ y = c.v.y;
    const bool folded = c.v.sval_shift != nullptr;  // the product already holds sigma q
    double2 acc = make_double2(0.0, 0.0);
    auto epi = [&](unsigned r, double ax) {
        const double qr = HBK_LD(G, q, r);
        const double yv = folded ? ax : fma(sig, qr, ax);
        y[r] = yv;
        acc.x = fma(qr, qr, acc.x);
        acc.y = fma(qr, yv, acc.y);
    };
    spmv_rows<FMT>(c.A, q, epi, g);
    acc = block_sum2(acc, red);
    if (threadIdx.x == 0) {
        c.sh.partials[g.b()] = acc.x;
        c.sh.partials[HBK_MAX_GRID + g.b()] = acc.y;
    }
    if (take_ticket(c.sh.counters + 1, g.nb())) {
        const double qq = sum_partials(c.sh.partials, g.nb(), red);
        const double qy = sum_partials(c.sh.partials + HBK_MAX_GRID, g.nb(), red);
        if (threadIdx.x == 0) {
            const int k = sc->k;
            const double w = dvd(qq, qy);
            sc->qq = qq;
            sc->qy = qy;
            c.sh.w_hist[k] = w;
            sc->omega = w;
            sc->rr_hat_old = sc->rr_hat;
            if (!fin(w) || w == 0.0) {
                sc->status |= HBK_ST_BREAKDOWN;
                sc->finished = 1;
            }
            c.sh.counters[1] = 0;
        }
    }
}
template <int FMT>
__global__ void __launch_bounds__(NT) k_seed_y(Ctx c) { seed_y_body<FMT>(c, HwGrid()); }
template <>
__global__ void __launch_bounds__(NT, HBK_HYB_MINB) k_seed_y<HBK_FMT_HYB>(Ctx c) {
    seed_y_body<HBK_FMT_HYB>(c, HwGrid());
}

// ---------------------------------------------------------------------------
// End of the seed step, run by the last block of K4: beta, the shift
// recurrences (src/solver_dynamic.c:243-253), the convergence test
// (:278-303) and the seed switch (:312-359).
__device__ void seed_step_scalars(const Ctx &c, double rr, double rrh) {
    __shared__ double s_bk;
    __shared__ int s_ok, s_sw, s_t, s_nconv, s_nfail;
    __shared__ double s_best[NW];
    __shared__ int s_bidx[NW];
    hbk_scalars *sc = c.sh.sc;
    const hbk_shifts &S = c.sh;
    const int k = sc->k, seed = sc->seed, m = S.m, kcap = S.kcap;
    const int deferred = c.v.deferred;
    if (threadIdx.x == 0) {
        sc->rr = rr;
        if (k < kcap) S.rr_hist[k] = rr;
        const double bk = mul(dvd(S.a_hist[k], S.w_hist[k]), dvd(rrh, sc->rr_hat_old));
        S.b_hist[k] = bk;
        sc->beta = bk;
        sc->rr_hat = rrh;
        s_bk = bk;
        s_ok = fin(bk);
        s_nfail = 0;
        if (!s_ok) {
            sc->status |= HBK_ST_BREAKDOWN;
            sc->finished = 1;
        }
    }
    __syncthreads();
    if (!s_ok) return;
    const double ak = S.a_hist[k], wk = S.w_hist[k], bk = s_bk;
    const double c_prev = mul(dvd(S.b_hist[k - 1], S.a_hist[k - 1]), ak);
    const double sig_s = S.sigma[seed];

    // (1) per-shift recurrences and this iteration's vector coefficients
    for (int j = threadIdx.x; j < m; j += NT) {
        double *co = S.coef + (size_t)j * HBK_NCOEF;
        if (j == seed) {
            // the seed as a system of its own (deferred mode): pi = zeta = 1,
            // shift 0.  Its x is not carried in coefficient form: K4 adds
            // alpha p_s + omega q to its row of X directly, with the
            // materialised p_s, as the reference's seed step does
            // (src/solver_dynamic.c:156-210).  In coefficient form p_s would enter
            // through s = (r_{k-1} - q) / alpha, which cancels when a step makes
            // little progress; its p coefficients stay (needed after a switch).
            co[0] = 0.0;
            co[1] = 0.0;
            co[2] = dvd(wk, ak);
            co[3] = -dvd(wk, ak);
            co[4] = bk;
            co[5] = 1.0;
            continue;
        }
        if (S.done[j]) continue;
        double *pij = S.pi + (size_t)j * kcap;
        const double d = sub(sig_s, S.sigma[j]);
        const double pik1 = pij[k - 1];
        const double eta = sub(mul(c_prev, S.eta[j]), mul(mul(d, ak), pik1));
        const double pik = add(eta, pik1);
        const double den = sub(1.0, mul(wk, d));
        const double aj = mul(dvd(pik1, pik), ak);
        const double wj = dvd(wk, den);
        const double z = S.zeta[j];
        double cn[6];
        cn[0] = dvd(wj, mul(pik, z));
        cn[1] = aj;
        cn[2] = dvd(wj, mul(mul(aj, z), pik));
        cn[3] = dvd(-wj, mul(mul(aj, z), pik1));
        const double zn = mul(den, z);
        const double rp = dvd(pik1, pik);
        cn[4] = mul(mul(rp, rp), bk);
        cn[5] = dvd(1.0, mul(pik, zn));
        // Shift breakdown (the reference never tests for it and carries the
        // inf or nan into x_j): pi_k = 0, 1 - omega_k d = 0, or any scalar of
        // the update not finite.  The shift stops at its last finite iterate,
        // counts as finished so the others run on, and records -k.
        bool ok = pik != 0.0 && den != 0.0 && fin(eta) && fin(zn);
#pragma unroll
        for (int t = 0; t < 6; t++) ok = ok && fin(cn[t]);
        if (!ok) {
            S.done[j] = 1;
            S.conv_k[j] = -k;
            atomicAdd(&s_nfail, 1);
            continue;
        }
        pij[k] = pik;
        S.eta[j] = eta;
        S.zeta[j] = zn;
#pragma unroll
        for (int t = 0; t < 6; t++) co[t] = cn[t];
    }
    __syncthreads();

    // (2) the systems updated this iteration, in index order
    if (threadIdx.x == 0) {
        int na = 0;
        if (deferred) S.act_list[na++] = seed;
        for (int j = 0; j < m; j++)
            if (j != seed && !S.done[j]) S.act_list[na++] = j;
        sc->n_active = na;
        if (k < kcap) S.act_hist[k] = na - deferred;
    }
    __syncthreads();

    // (3) convergence test on the recursive residual; argmax of |1/(zeta pi)|
    //     over the systems still running, strict '>' from 1.0 (lowest index
    //     wins an exact tie)
    const double thr = mul(mul(sc->tol, sc->tol), sc->bb);
    double best = 1.0;
    int bidx = -1, nconv = 0;
    for (int j = threadIdx.x; j < m; j += NT) {
        if (S.done[j]) continue;
        const double a = (j == seed) ? 1.0 : fabs(dvd(1.0, mul(S.zeta[j], S.pi[(size_t)j * kcap + k])));
        if (mul(mul(a, a), rr) <= thr) {
            S.done[j] = 1;
            S.conv_k[j] = k;
            nconv++;
        } else if (a > best) {
            best = a;
            bidx = j;
        }
    }
    // block argmax: larger value wins, lower index on ties
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (oi >= 0 && (bidx < 0 || ob > best || (ob == best && oi < bidx))) {
            best = ob;
            bidx = oi;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        s_best[threadIdx.x >> 5] = best;
        s_bidx[threadIdx.x >> 5] = bidx;
    }
    if (threadIdx.x == 0) s_nconv = 0;
    __syncthreads();
    if (nconv) atomicAdd(&s_nconv, nconv);
    __syncthreads();
    if (threadIdx.x == 0) {
        double bb2 = 1.0;
        int bi = -1;
        for (int w = 0; w < NW; w++) {
            const int oi = s_bidx[w];
            const double ob = s_best[w];
            if (oi >= 0 && (bi < 0 || ob > bb2 || (ob == bb2 && oi < bi))) {
                bb2 = ob;
                bi = oi;
            }
        }
        if (bi >= 0) sc->max_sigma = bi;
        sc->n_done += s_nconv + s_nfail;
        if (s_nfail) sc->status |= HBK_ST_SHIFT_FAIL;
        s_sw = (sc->switching && S.done[seed] && sc->n_done < m) ? 1 : 0;
        s_t = sc->max_sigma;
        sc->next_seed = s_sw ? s_t : seed;
        sc->switched = s_sw;
        sc->r_scale = 1.0;
    }
    __syncthreads();
    if (!s_sw) return;

    // (4) seed switch to t: rescale the seed history, rescale r (K5), replay
    //     eta/pi/zeta of every running shift relative to sigma_t
    const int t = s_t;
    const double *pit = S.pi + (size_t)t * kcap;
    const double dst = sub(sig_s, S.sigma[t]);
    if (threadIdx.x == 0) sc->r_scale = dvd(1.0, mul(S.zeta[t], pit[k]));
    for (int i = 1 + threadIdx.x; i <= k; i += NT) {
        const double rp = dvd(pit[i - 1], pit[i]);
        S.a_hist[i] = mul(rp, S.a_hist[i]);
        S.b_hist[i] = mul(mul(rp, rp), S.b_hist[i]);
        S.w_hist[i] = dvd(S.w_hist[i], sub(1.0, mul(S.w_hist[i], dst)));
    }
    __syncthreads();
    for (int i = 1 + threadIdx.x; i <= k; i += NT) S.ratio[i] = mul(dvd(S.b_hist[i - 1], S.a_hist[i - 1]), S.a_hist[i]);
    __syncthreads();
    const double sig_t = S.sigma[t];
    for (int j = threadIdx.x; j < m; j += NT) {
        if (S.done[j] || j == t) {
            S.eta[j] = 0.0;
            S.zeta[j] = 1.0;
            continue;
        }
        double *pij = S.pi + (size_t)j * kcap;
        const double d = sub(sig_t, S.sigma[j]);
        double e = 0.0, z = 1.0, pprev = pij[0];
        for (int i = 1; i <= k; i++) {
            e = sub(mul(S.ratio[i], e), mul(mul(d, S.a_hist[i]), pprev));
            const double pc = add(e, pprev);
            pij[i] = pc;
            z = mul(sub(1.0, mul(S.w_hist[i], d)), z);
            pprev = pc;
        }
        S.eta[j] = e;
        S.zeta[j] = z;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        S.eta[t] = 0.0;
        S.zeta[t] = 1.0;
        if (sc->n_sw < m) {
            S.sw_k[sc->n_sw] = k;
            S.sw_seed[sc->n_sw] = t;
        }
        sc->n_sw++;
    }
}

// K4: x_s += alpha p_s + omega q ; r_k = q - omega y ; (r,r), (r^,r)
// (at least 4 CTAs per SM: the streaming loop needs the warps; the scalar
// stage that runs in one CTA per iteration may spill)
template <class G>
__device__ __forceinline__ void seed_update_body(const Ctx &c, const G &g) {
    __shared__ double sh[2 * NW];
    __shared__ unsigned long long smx[NW];
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const double a = sc->alpha, w = sc->omega;
    const int seed = sc->seed;
    const unsigned n = c.v.n;
    const double *__restrict__ ps = seed_p(c, seed);
    const double *__restrict__ q = vec_q(c, sc);
    const double *__restrict__ y = c.v.y;
    const double *__restrict__ rh = c.v.r_hat;
    double *__restrict__ rn = vec_r_new(c, sc);
    double2 acc = make_double2(0.0, 0.0);
    unsigned long long mx = 0;
    // the seed's x in both shift modes (in deferred mode its x coefficients
    // are kept at zero, so the basis flushes leave it as it is; there x_j are
    // panel-major)
    const bool dm = c.v.deferred != 0;
    double *__restrict__ xrow = dm ? c.v.Xp : c.v.X + (size_t)seed * ldn(n);
    const int pm = c.v.pm;
    for (size_t i = g.b() * (size_t)NT + threadIdx.x; i < n; i += (size_t)g.nb() * NT) {
        const double qi = HBK_LD(G, q, i);
        double *xi = dm ? xrow + panel_idx(seed, (unsigned)i, pm) : xrow + i;
        *xi = fma(w, qi, fma(a, HBK_LD(G, ps, i), HBK_LD(G, xi, 0)));
        const double r = fma(-w, HBK_LD(G, y, i), qi);
        rn[i] = r;
        acc.x = fma(r, r, acc.x);
        acc.y = fma(HBK_LD(G, rh, i), r, acc.y);
        const unsigned long long b = abs_bits(r);
        mx = b > mx ? b : mx;
    }
    if (c.v.slot_max) block_max_to(mx, smx, c.v.slot_max + (size_t)(sc->slots + 1) * HBK_SLOT_SPREAD);  // r_k
    acc = block_sum2(acc, sh);
    if (threadIdx.x == 0) {
        c.sh.partials[g.b()] = acc.x;
        c.sh.partials[HBK_MAX_GRID + g.b()] = acc.y;
    }
    if (take_ticket(c.sh.counters + 2, g.nb())) {
        const double rr = sum_partials(c.sh.partials, g.nb(), sh);
        const double rrh = sum_partials(c.sh.partials + HBK_MAX_GRID, g.nb(), sh);
        seed_step_scalars(c, rr, rrh);
        if (threadIdx.x == 0) c.sh.counters[2] = 0;
    }
}
__global__ void __launch_bounds__(NT, 4) k_seed_update(Ctx c) { seed_update_body(c, HwGrid()); }

// End of an iteration (one thread): apply the switch, advance k, test the loop.
__device__ void finish_iteration(const Ctx &c, hbk_scalars *sc, double rrh_scaled) {
    if (sc->switched) {
        sc->rr_hat = rrh_scaled;
        sc->seed = sc->next_seed;
        sc->switched = 0;
        if (c.v.deferred) {
            sc->slot_r_old = sc->slots + 2;  // the rescaled r_k
            sc->slots += 3;
            sc->need_ps = 1;
        }
    } else if (c.v.deferred) {
        sc->slot_r_old = sc->slots + 1;
        sc->slots += 2;
    }
    sc->k += 1;
    if (sc->n_done >= sc->m || sc->k >= sc->kcap) sc->finished = 1;
    if (c.v.deferred && !sc->finished && sc->slots + 3 > sc->slot_cap) {
        sc->status |= HBK_ST_BASIS_FULL;
        sc->finished = 1;  // the host flushes the basis and resumes
    }
}

// K5 (incremental): p_s, then every running shift's x_j and p_j in one pass
// over q, r_{k-1}, r_k (src/solver_dynamic.c:208-210, :248-255)
template <int MAXS, class G>
__device__ __forceinline__ void shift_update_body(const Ctx &c, const G &g) {
    __shared__ double s_co[MAXS * 6];
    __shared__ int s_j[MAXS];
    __shared__ double sh[NW];
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const int seed = sc->seed, na = sc->n_active, k = sc->k;
    const double bk = sc->beta, wk = sc->omega, bw = -mul(bk, wk);
    const int sw = sc->switched;
    const double rsc = sc->r_scale;
    const unsigned n = c.v.n;
    const size_t ld = ldn(n);
    double *__restrict__ ps = c.v.P + (size_t)seed * ld;
    const double *__restrict__ q = c.v.q;
    const double *__restrict__ s = c.v.s;
    const double *__restrict__ ro = c.v.rbuf[(k - 1) & 1];
    double *__restrict__ rn = c.v.rbuf[k & 1];
    const double *__restrict__ rh = c.v.r_hat;
    double acc = 0.0;
    for (int base = 0; base < na || base == 0; base += MAXS) {
        const int cnt = min(MAXS, na - base);
        for (int a = threadIdx.x; a < cnt; a += NT) {
            const int j = c.sh.act_list[base + a];
            s_j[a] = j;
            const double *co = c.sh.coef + (size_t)j * HBK_NCOEF;
#pragma unroll
            for (int t = 0; t < 6; t++) s_co[a * 6 + t] = co[t];
        }
        __syncthreads();
        for (size_t i = g.b() * (size_t)NT + threadIdx.x; i < n; i += (size_t)g.nb() * NT) {
            const double qi = HBK_LD(G, q, i), oi = HBK_LD(G, ro, i), ri = HBK_LD(G, rn, i);
            if (base == 0) ps[i] = fma(bw, HBK_LD(G, s, i), fma(bk, HBK_LD(G, ps, i), ri));
            for (int a = 0; a < cnt; a++) {
                const double *co = s_co + a * 6;
                double *xj = c.v.X + (size_t)s_j[a] * ld;
                double *pj = c.v.P + (size_t)s_j[a] * ld;
                double x = HBK_LD(G, xj, i), p = HBK_LD(G, pj, i);
                x = fma(co[0], qi, x);
                x = fma(co[1], p, x);
                p = fma(co[2], qi, p);
                p = fma(co[3], oi, p);
                p = co[4] * p;
                p = fma(co[5], ri, p);
                xj[i] = x;
                pj[i] = p;
            }
            if (sw && base + MAXS >= na) {
                const double rs = ri * rsc;
                rn[i] = rs;
                acc = fma(HBK_LD(G, rh, i), rs, acc);
            }
        }
        __syncthreads();
        if (na <= MAXS) break;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) c.sh.partials[g.b()] = acc;
    if (take_ticket(c.sh.counters + 3, g.nb())) {
        const double rrh = sum_partials(c.sh.partials, g.nb(), sh);
        if (threadIdx.x == 0) {
            finish_iteration(c, sc, rrh);
            c.sh.counters[3] = 0;
        }
    }
}
template <int MAXS>
__global__ void __launch_bounds__(NT) k_shift_update(Ctx c) { shift_update_body<MAXS>(c, HwGrid()); }

// K5 (deferred): p_s update; on a switch the rescaled r_k goes to a new slot
template <class G>
__device__ __forceinline__ void seed_p_deferred_body(const Ctx &c, const G &g) {
    __shared__ double sh[NW];
    __shared__ unsigned long long smx[NW];
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const double bk = sc->beta, bw = -mul(bk, sc->omega);
    const int sw = sc->switched;
    const double rsc = sc->r_scale;
    const unsigned n = c.v.n;
    const size_t ld = ldn(n);
    double *__restrict__ ps = c.v.ps;
    const double *__restrict__ s = c.v.s;
    const double *__restrict__ rn = c.v.V + (size_t)(sc->slots + 1) * ld;
    double *__restrict__ rsl = c.v.V + (size_t)(sc->slots + 2) * ld;
    const double *__restrict__ rh = c.v.r_hat;
    double acc = 0.0;
    unsigned long long mx = 0;
    for (size_t i = g.b() * (size_t)NT + threadIdx.x; i < n; i += (size_t)g.nb() * NT) {
        const double ri = HBK_LD(G, rn, i);
        ps[i] = fma(bw, HBK_LD(G, s, i), fma(bk, HBK_LD(G, ps, i), ri));
        if (sw) {
            const double rs = ri * rsc;
            rsl[i] = rs;
            acc = fma(HBK_LD(G, rh, i), rs, acc);
            const unsigned long long b = abs_bits(rs);
            mx = b > mx ? b : mx;
        }
    }
    if (!sw) return;  // uniform: the reduction is needed only after a switch
    if (c.v.slot_max) block_max_to(mx, smx, c.v.slot_max + (size_t)(sc->slots + 2) * HBK_SLOT_SPREAD);  // rescaled r_k
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) c.sh.partials[g.b()] = acc;
    if (take_ticket(c.sh.counters + 3, g.nb())) {
        const double rrh = sum_partials(c.sh.partials, g.nb(), sh);
        if (threadIdx.x == 0) {
            sc->rs_switch = rrh;
            c.sh.counters[3] = 0;
        }
    }
}
__global__ void __launch_bounds__(NT) k_seed_p_deferred(Ctx c) { seed_p_deferred_body(c, HwGrid()); }

// K6 (deferred): coefficient update of every running system over the basis
// slots in use, then the end-of-iteration bookkeeping.  Per coefficient the
// operations follow the vector update's order (x += c0 q; x += c1 p;
// p += c2 q; p += c3 r_{k-1}; p *= beta_j; p += c5 r_k).
template <class G>
__device__ __forceinline__ void coef_update_body(const Ctx &c, const G &g) {
    hbk_scalars *sc = c.sh.sc;
    if (stopped(sc)) return;
    const int na = sc->n_active;
    const int sq = sc->slots, sr = sc->slots + 1, so = sc->slot_r_old;
    const int L = sc->slots + 2;
    const int cap = c.v.slot_cap;
    const size_t tot = (size_t)na * L;
    for (size_t it = g.b() * (size_t)NT + threadIdx.x; it < tot; it += (size_t)g.nb() * NT) {
        const int a = (int)(it / L), i = (int)(it % L);
        const int j = HBK_LD(G, c.sh.act_list, a);
        const double *co = c.sh.coef + (size_t)j * HBK_NCOEF;
        double *xc = c.v.Xc + (size_t)j * cap + i;
        double *pc = c.v.Pc + (size_t)j * cap + i;
        double x = HBK_LD(G, xc, 0), p = HBK_LD(G, pc, 0);
        if (i == sq) x = x + co[0];
        x = fma(co[1], p, x);
        if (i == sq) p = p + co[2];
        if (i == so) p = p + co[3];
        p = co[4] * p;
        if (i == sr) p = p + co[5];
        *xc = x;
        *pc = p;
        if (i == 0) {
            double *ow = c.v.own + 2 * (size_t)j;
            ow[0] = fma(co[1], HBK_LD(G, ow, 1), HBK_LD(G, ow, 0));
            ow[1] = co[4] * HBK_LD(G, ow, 1);
            c.sh.lslot[j] = L;
        }
    }
    if (take_ticket(c.sh.counters + 4, g.nb())) {
        if (threadIdx.x == 0) {
            finish_iteration(c, sc, sc->rs_switch);
            c.sh.counters[4] = 0;
        }
    }
}
__global__ void __launch_bounds__(NT) k_coef_update(Ctx c) { coef_update_body(c, HwGrid()); }

// K7 (deferred): after a switch, the new seed's p = own term + Pc[t] . V
template <class G>
__device__ __forceinline__ void materialize_ps_body(const Ctx &c, const G &g) {
    __shared__ double s_c[1024];
    hbk_scalars *sc = c.sh.sc;
    if (!__ldcg(&sc->need_ps)) return;
    const int t = sc->seed;
    const int L = HBK_LD(G, c.sh.lslot, t);
    const unsigned n = c.v.n;
    const size_t ld = ldn(n);
    const double *pc = c.v.Pc + (size_t)t * c.v.slot_cap;
    const double rho = HBK_LD(G, c.v.own, 2 * (size_t)t + 1);
    const double *pmat = c.v.Pmat;  // panel-major
    for (size_t i0 = (size_t)g.b() * NT; i0 < n; i0 += (size_t)g.nb() * NT) {
        const size_t i = i0 + threadIdx.x;
        double acc = (pmat && i < n) ? rho * pmat[panel_idx(t, (unsigned)i, c.v.pm)] : 0.0;
        for (int l0 = 0; l0 < L; l0 += 1024) {
            const int cnt = min(1024, L - l0);
            __syncthreads();
            for (int l = threadIdx.x; l < cnt; l += NT) s_c[l] = HBK_LD(G, pc, l0 + l);
            __syncthreads();
            if (i < n)
                for (int l = 0; l < cnt; l++) acc = fma(s_c[l], HBK_LD(G, c.v.V, (size_t)(l0 + l) * ld + i), acc);
        }
        if (i < n) c.v.ps[i] = acc;
    }
    if (c.v.sval_shift) {  // the new seed's shift on the diagonal of the seed kernels' products
        const double sg = c.sh.sigma[t];
        for (size_t r = g.b() * (size_t)NT + threadIdx.x; r < n; r += (size_t)g.nb() * NT) {
            const unsigned long long d = c.v.sdiag[r];
            c.v.sval_shift[d] = c.v.sval_orig[d] + sg;
        }
    }
    if (take_ticket(c.sh.counters + 5, g.nb())) {
        if (threadIdx.x == 0) {
            sc->need_ps = 0;
            c.sh.counters[5] = 0;
        }
    }
}
__global__ void __launch_bounds__(NT) k_materialize_ps(Ctx c) { materialize_ps_body(c, HwGrid()); }

// Flush: X_j += xi_j Pmat_j + Xc_j . V ; when keep_p, Pmat_j = rho_j Pmat_j + Pc_j . V.
// Each thread owns one row and GROUP systems; coefficients are staged in
// shared memory per chunk of slots.  FP64 FMA-bound by design: it is the
// only place the per-shift solutions are formed.
constexpr int GROUP = 16;
constexpr int LCH = 64;
__global__ void __launch_bounds__(NT) k_flush(Ctx c, int keep_p, int which) {
    __shared__ double s_c[GROUP * LCH];
    const unsigned n = c.v.n;
    const size_t ld = ldn(n);
    const int m = c.sh.m, cap = c.v.slot_cap;
    const int j0 = blockIdx.y * GROUP;
    const int g = min(GROUP, m - j0);
    int L = 0;
    for (int t = 0; t < g; t++) L = max(L, c.sh.lslot[j0 + t]);
    const double *coef = which == 0 ? c.v.Xc : c.v.Pc;
    double *out = which == 0 ? c.v.Xp : c.v.Pmat;  // panel-major
    const int pm = c.v.pm;
    for (size_t i0 = (size_t)blockIdx.x * NT; i0 < n; i0 += (size_t)gridDim.x * NT) {
        const size_t i = i0 + threadIdx.x;
        double acc[GROUP];
#pragma unroll
        for (int t = 0; t < GROUP; t++) {
            acc[t] = 0.0;
            if (t < g && i < n) {
                const int j = j0 + t;
                const size_t pi = panel_idx(j, (unsigned)i, pm);
                const double *pmat = c.v.Pmat;
                if (which == 0) {
                    acc[t] = c.v.Xp[pi];
                    if (pmat) acc[t] = fma(c.v.own[2 * (size_t)j], pmat[pi], acc[t]);
                } else if (pmat) {
                    acc[t] = c.v.own[2 * (size_t)j + 1] * pmat[pi];
                }
            }
        }
        for (int l0 = 0; l0 < L; l0 += LCH) {
            const int cnt = min(LCH, L - l0);
            __syncthreads();
            for (int e = threadIdx.x; e < GROUP * LCH; e += NT) {
                const int t = e / LCH, l = e % LCH;
                s_c[e] = (t < g && l < cnt) ? coef[(size_t)(j0 + t) * cap + l0 + l] : 0.0;
            }
            __syncthreads();
            if (i < n) {
                for (int l = 0; l < cnt; l++) {
                    const double v = c.v.V[(size_t)(l0 + l) * ld + i];
#pragma unroll
                    for (int t = 0; t < GROUP; t++) acc[t] = fma(s_c[t * LCH + l], v, acc[t]);
                }
            }
        }
        if (i < n) {
#pragma unroll
            for (int t = 0; t < GROUP; t++)
                if (t < g) out[panel_idx(j0 + t, (unsigned)i, pm)] = acc[t];
        }
    }
    (void)keep_p;
}

// after a flush: reset the coefficients, own = (0, 1), slot 0 = r_{k-1}
__global__ void __launch_bounds__(NT) k_flush_reset(Ctx c, int keep_p) {
    hbk_scalars *sc = c.sh.sc;
    const int m = c.sh.m, cap = c.v.slot_cap;
    const unsigned n = c.v.n;
    const size_t ld = ldn(n);
    const int so = sc->slot_r_old;
    const size_t tot = (size_t)m * cap;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < tot; i += (size_t)gridDim.x * NT) {
        c.v.Xc[i] = 0.0;
        c.v.Pc[i] = 0.0;
    }
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < (size_t)m; i += (size_t)gridDim.x * NT) {
        c.v.own[2 * i] = 0.0;
        c.v.own[2 * i + 1] = keep_p ? 1.0 : 0.0;
        c.sh.lslot[i] = 1;
    }
    if (so != 0)
        for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT)
            c.v.V[i] = c.v.V[(size_t)so * ld + i];
    if (c.v.slot_max) {
        // slot 0 takes the copied slot's maximum (one thread: no other thread
        // touches slots 0 and so); the others start empty
        const size_t tot_e = (size_t)cap * HBK_SLOT_SPREAD;
        for (size_t e = blockIdx.x * (size_t)NT + threadIdx.x; e < tot_e; e += (size_t)gridDim.x * NT) {
            const size_t l = e / HBK_SLOT_SPREAD;
            if (l != 0 && l != (size_t)so) c.v.slot_max[e] = 0;
        }
        if (blockIdx.x == 0 && threadIdx.x < HBK_SLOT_SPREAD && so != 0) {
            const size_t e0 = threadIdx.x, es = (size_t)so * HBK_SLOT_SPREAD + threadIdx.x;
            c.v.slot_max[e0] = c.v.slot_max[es];
            c.v.slot_max[es] = 0;
        }
    }
    if (take_ticket(c.sh.counters + 6)) {
        if (threadIdx.x == 0) {
            sc->slots = 1;
            sc->slot_r_old = 0;
            sc->status &= ~HBK_ST_BASIS_FULL;
            if (sc->n_done < sc->m && sc->k < sc->kcap && !(sc->status & HBK_ST_BREAKDOWN)) sc->finished = 0;
            c.sh.counters[6] = 0;
        }
    }
}

// out[0 .. HBK_SLOT_SPREAD) take the bits of max |x| (zeroed by the caller)
__global__ void __launch_bounds__(NT) k_absmax(const double *__restrict__ x, unsigned n, unsigned long long *out) {
    __shared__ unsigned long long smx[NW];
    unsigned long long mx = 0;
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT) {
        const unsigned long long b = abs_bits(x[i]);
        mx = b > mx ? b : mx;
    }
    block_max_to(mx, smx, out);
}

// End of a while-loop body in a CUDA graph: run again while the solve goes on
// (not finished: converged, at max_iter, broken down or waiting for a basis
// flush), and never more than loop_cap bodies per solve.
__global__ void k_loop_condition(hbk_scalars *sc, cudaGraphConditionalHandle cond, int loop_cap) {
    const int loops = ++sc->loops;
    cudaGraphSetConditional(cond, (!sc->finished && loops < loop_cap) ? 1u : 0u);
}

// x[i] = element i of system j of the panel-major Xp (runs of HBK_PANEL)
__global__ void __launch_bounds__(NT) k_panel_row(const double *__restrict__ Xp, int m, unsigned n, int j,
                                                  double *__restrict__ x) {
    for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < n; i += (size_t)gridDim.x * NT)
        x[i] = Xp[panel_idx(j, (unsigned)i, m)];
}

// X[j][i] = element i of system j of the panel-major Xp: one block per panel
// (m * HBK_PANEL values read contiguously, written as runs of HBK_PANEL)
__global__ void __launch_bounds__(NT) k_panel_to_rows(const double *__restrict__ Xp, int m, unsigned n,
                                                      double *__restrict__ X, size_t ld) {
    const unsigned per = (unsigned)m * HBK_PANEL;
    const size_t np = ((size_t)n + HBK_PANEL - 1) / HBK_PANEL;
    for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
        const double *src = Xp + p * per;
        const size_t i0 = p * HBK_PANEL;
        for (unsigned r = threadIdx.x; r < per; r += NT) {
            const unsigned j = r / HBK_PANEL, c = r - j * HBK_PANEL;
            if (i0 + c < n) X[(size_t)j * ld + i0 + c] = src[r];
        }
    }
}

// ---------------------------------------------------------------------------
// Many families in one persistent launch (SELL-32, either shift mode).
//
// Each family's rows are cut into virtual blocks of HBK_GROUP_ROWS rows; the
// CTAs of one cooperative launch take the virtual blocks of all families in
// turn (virtual block v goes to CTA v mod grid, so a family's rows stay on
// the same CTAs from step to step) and run, for every family at once, the
// same steps as the one-family kernels (K1..K5, and K6, K7 for the families
// in the deferred mode, with a virtual block in place of the launch's block:
// same partial sums, same last-block tickets and scalar stage per family).  A
// grid-wide barrier separates the steps.  Families stop one by one
// (converged, max_iter, breakdown) or pause with a full basis; their virtual
// blocks then return at once, and the launch ends when every family has
// stopped or paused (the host flushes the paused ones and launches again).
struct GroupFam {
    Ctx c;
    unsigned vb0, nvb;  // the family's virtual blocks [vb0, vb0 + nvb)
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier over every CTA of a cooperative launch: bar[0] counts arrivals,
// bar[1] is the generation (the last CTA to arrive resets the count and bumps
// it, with release order; the others wait for it with acquire loads).  A wait
// longer than HBK_GROUP_WAIT_NS sets *err; every CTA that sees *err leaves the
// wait, so the launch ends (with the error) instead of hanging.  Returns
// false in every thread of the CTA when the launch must stop.  withhold:
// this CTA waits without arriving (the bounded-wait test: every CTA then
// waits out the bound, and the launch ends with HBK_GROUP_ERR_WAIT).
__device__ bool grid_barrier(unsigned *bar, int *err, bool withhold = false) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = ld_acquire_u32(bar + 1);
        const unsigned arrived = withhold ? 0u : atom_add_acq_rel_u32(bar, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(bar, 0u);
            st_release_u32(bar + 1, gen + 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acquire_u32(bar + 1) == gen) {
                if (*(volatile int *)err) {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > HBK_GROUP_WAIT_NS) {
                    atomicExch(err, HBK_GROUP_ERR_WAIT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
        }
        s_ok = ok && *(volatile int *)err == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// step 5: the shift update (incremental) or the seed's p update (deferred)
template <int MAXS>
__device__ __forceinline__ void step5_body(const Ctx &c, const VGrid &g) {
    if (c.v.deferred) seed_p_deferred_body(c, g);
    else shift_update_body<MAXS>(c, g);
}
__device__ __forceinline__ void coef_update_if_deferred(const Ctx &c, const VGrid &g) {
    if (c.v.deferred) coef_update_body(c, g);
}
__device__ __forceinline__ void materialize_if_deferred(const Ctx &c, const VGrid &g) {
    if (c.v.deferred) materialize_ps_body(c, g);
}

// (3 CTAs per SM: the register cap costs a few spills in the scalar stage)
template <int MAXS>
__global__ void __launch_bounds__(NT, 3) k_group(const GroupFam *__restrict__ fams, int nf,
                                                 const unsigned *__restrict__ vb_fam, unsigned nvb, unsigned *bar,
                                                 int *err, int iter_cap, int any_deferred, int withhold) {
#define HBK_GROUP_STEP(body)                                                       \
    for (unsigned vb = blockIdx.x; vb < nvb; vb += gridDim.x) {                    \
        const GroupFam &F = fams[vb_fam[vb]];                                      \
        body(F.c, VGrid{vb - F.vb0, F.nvb});                                       \
    }                                                                              \
    if (!grid_barrier(bar, err)) return;
    for (int it = 0; it <= iter_cap; ++it) {
        // any family still running?  (read between two barriers: no step
        // writes a family's stop flag meanwhile, so every CTA sees the same)
        int alive = 0;
        for (int f = threadIdx.x; f < nf; f += NT) alive |= __ldcg(&fams[f].c.sh.sc->finished) == 0;
        alive = __syncthreads_or(alive);
        if (!grid_barrier(bar, err, withhold && it == 0 && blockIdx.x == 0) || !alive) return;
        HBK_GROUP_STEP(seed_s_body<HBK_FMT_SELL>)
        HBK_GROUP_STEP(seed_q_body)
        HBK_GROUP_STEP(seed_y_body<HBK_FMT_SELL>)
        HBK_GROUP_STEP(seed_update_body)
        HBK_GROUP_STEP(step5_body<MAXS>)
        if (any_deferred) {
            HBK_GROUP_STEP(coef_update_if_deferred)
            HBK_GROUP_STEP(materialize_if_deferred)
        }
    }
#undef HBK_GROUP_STEP
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(err, HBK_GROUP_ERR_CAP);
}

}  // namespace

extern "C" {

int hbk_panel_row(const double *Xp, int m, unsigned n, int j, double *x, cudaStream_t st) {
    if (n == 0 || j < 0 || j >= m) return 0;
    k_panel_row<<<grid_for(n, 4), NT, 0, st>>>(Xp, m, n, j, x);
    return (int)cudaGetLastError();
}

int hbk_panel_to_rows(const double *Xp, int m, unsigned n, double *X, size_t ld, cudaStream_t st) {
    if (m <= 0 || n == 0) return 0;
    const size_t np = ((size_t)n + HBK_PANEL - 1) / HBK_PANEL;
    k_panel_to_rows<<<(unsigned)(np < 4864 ? np : 4864), NT, 0, st>>>(Xp, m, n, X, ld);
    return (int)cudaGetLastError();
}

static Ctx make_ctx(const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh) {
    Ctx c;
    c.A = *A;
    c.v = *v;
    c.sh = *sh;
    // the seed shift sits on the diagonal of a private copy of the SELL-32
    // values: only while the matrix is in that form and the copy was made from it
    if (c.v.sval_shift && c.A.fmt == HBK_FMT_SELL && c.v.deferred && c.A.sval == c.v.sval_orig)
        c.A.sval = c.v.sval_shift;
    else
        c.v.sval_shift = nullptr;
    return c;
}

int hbk_fused_init(const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, const double *b, int seed,
                   double tol, cudaStream_t st) {
    Ctx c = make_ctx(A, v, sh);
    const unsigned n = v->n;
    const size_t ld = ((size_t)n + 31) / 32 * 32;
    int e;
    if ((e = hbk_copy(n, b, v->r_hat, st))) return e;
    if ((e = hbk_dot(n, b, b, sh->partials, sh->counters + 7, &sh->sc->bb, st))) return e;
    if (!v->deferred) {
        if ((e = hbk_copy(n, b, v->rbuf[0], st))) return e;
        for (int j = 0; j < sh->m; j++) {
            if ((e = hbk_copy(n, b, v->P + (size_t)j * ld, st))) return e;
        }
    } else {
        if ((e = hbk_copy(n, b, v->V, st))) return e;
        if ((e = hbk_copy(n, b, v->ps, st))) return e;
        if (v->sval_shift && A->fmt == HBK_FMT_SELL && A->sval == v->sval_orig &&
            (e = hbk_fold_diag(n, A->sval, A->sell_len, v->sdiag, sh->sigma + seed, v->sval_shift, st)))
            return e;
        if (v->slot_max) {
            if ((e = (int)cudaMemsetAsync(v->slot_max, 0,
                                          sizeof(unsigned long long) * (size_t)v->slot_cap * HBK_SLOT_SPREAD, st)))
                return e;
            k_absmax<<<grid_for(n ? n : 1, 4), NT, 0, st>>>(b, n, v->slot_max);  // slot 0 = b
            if ((e = (int)cudaGetLastError())) return e;
        }
        k_init_coef<<<grid_for((unsigned)((size_t)sh->m * v->slot_cap), 1), NT, 0, st>>>(c);
        if ((e = (int)cudaGetLastError())) return e;
    }
    if (v->deferred) {
        if ((e = (int)cudaMemsetAsync(v->Xp, 0, sizeof(double) * hbk_panel_elems(n, v->pm), st))) return e;
    } else if ((e = (int)cudaMemsetAsync(v->X, 0, sizeof(double) * ld * (size_t)sh->m, st))) {
        return e;
    }
    k_init<<<1, NT, 0, st>>>(c, seed, tol);
    return (int)cudaGetLastError();
}

int hbk_hyb_wave_fused(void) {
    const int a = wave_grid<k_seed_s<HBK_FMT_HYB>>(HBK_MAX_GRID), b = wave_grid<k_seed_y<HBK_FMT_HYB>>(HBK_MAX_GRID);
    return a < b ? a : b;
}

int hbk_fused_iteration(const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, cudaStream_t st) {
    Ctx c = make_ctx(A, v, sh);
    const int gv = grid_for(v->n, 2);
    // every kernel here is a grid-stride loop: launch at most one wave of it
    if (A->fmt == HBK_FMT_SELL) {
        k_seed_s<HBK_FMT_SELL><<<wave_grid<k_seed_s<HBK_FMT_SELL>>(A->grid), NT, 0, st>>>(c);
        k_seed_q<<<wave_grid<k_seed_q>(gv), NT, 0, st>>>(c);
        k_seed_y<HBK_FMT_SELL><<<wave_grid<k_seed_y<HBK_FMT_SELL>>(A->grid), NT, 0, st>>>(c);
    } else if (A->fmt == HBK_FMT_MERGE) {
        k_seed_s<HBK_FMT_MERGE><<<wave_grid<k_seed_s<HBK_FMT_MERGE>>(A->grid), NT, 0, st>>>(c);
        k_seed_q<<<wave_grid<k_seed_q>(gv), NT, 0, st>>>(c);
        k_seed_y<HBK_FMT_MERGE><<<wave_grid<k_seed_y<HBK_FMT_MERGE>>(A->grid), NT, 0, st>>>(c);
    } else if (A->fmt == HBK_FMT_HYB) {
        k_seed_s<HBK_FMT_HYB><<<wave_grid<k_seed_s<HBK_FMT_HYB>>(A->grid), NT, 0, st>>>(c);
        k_seed_q<<<wave_grid<k_seed_q>(gv), NT, 0, st>>>(c);
        k_seed_y<HBK_FMT_HYB><<<wave_grid<k_seed_y<HBK_FMT_HYB>>(A->grid), NT, 0, st>>>(c);
    } else {
        k_seed_s<HBK_FMT_TILE><<<wave_grid<k_seed_s<HBK_FMT_TILE>>(A->grid), NT, 0, st>>>(c);
        k_seed_q<<<wave_grid<k_seed_q>(gv), NT, 0, st>>>(c);
        k_seed_y<HBK_FMT_TILE><<<wave_grid<k_seed_y<HBK_FMT_TILE>>(A->grid), NT, 0, st>>>(c);
    }
    k_seed_update<<<wave_grid<k_seed_update>(gv), NT, 0, st>>>(c);
    if (!v->deferred) {
        // one element per thread: the update is FP64-bound (6 operations per
        // element and running shift), so on small systems it wants every SM's
        // FP64 pipe, not the two elements per thread of the streaming kernels
        k_shift_update<64><<<wave_grid<k_shift_update<64>>(grid_for(v->n, 1)), NT, 0, st>>>(c);
    } else {
        k_seed_p_deferred<<<wave_grid<k_seed_p_deferred>(gv), NT, 0, st>>>(c);
        k_coef_update<<<grid_for((unsigned)((size_t)sh->m * v->slot_cap), 1), NT, 0, st>>>(c);
        k_materialize_ps<<<wave_grid<k_materialize_ps>(gv), NT, 0, st>>>(c);
    }
    return (int)cudaGetLastError();
}

// the next shared launch's CTA 0 withholds its first barrier arrival (one
// shot; for the test of the bounded wait)
static int g_group_withhold = 0;
void hbk_group_test_withhold(int on) { g_group_withhold = on ? 1 : 0; }

static unsigned group_vblocks(unsigned n, unsigned rows) {
    if (rows == 0) rows = HBK_GROUP_ROWS;
    const unsigned v = (n + rows - 1) / rows;
    return v < 1 ? 1 : (v > HBK_MAX_GRID ? HBK_MAX_GRID : v);
}

static const size_t kGroupHead = 256;  // barrier words and the error flag

static size_t group_bytes(int nf, size_t nvb) {
    return kGroupHead + ((sizeof(GroupFam) * (size_t)nf + 255) / 256) * 256 + sizeof(unsigned) * nvb;
}

size_t hbk_group_ws_bytes(int nf, const hbk_vectors *v, unsigned rows_per_vb) {
    size_t nvb = 0;
    for (int f = 0; f < nf; ++f) nvb += group_vblocks(v[f].n, rows_per_vb);
    return group_bytes(nf, nvb);
}

int hbk_group_ctas(int max_ctas) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_group<64>, NT, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int one_wave = per_sm * sm_count();
    return max_ctas > 0 && max_ctas < one_wave ? max_ctas : one_wave;
}

int hbk_group_run(int nf, const hbk_matrix *A, const hbk_vectors *v, const hbk_shifts *sh, int iter_cap, int max_ctas,
                  unsigned rows_per_vb, void *ws, size_t ws_bytes, int *err_out, cudaStream_t st) {
    *err_out = 0;
    if (nf <= 0) return 0;
    int dev = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return (int)cudaErrorNotSupported;
    std::vector<GroupFam> tab((size_t)nf);
    std::vector<unsigned> map;
    int any_deferred = 0;
    for (int f = 0; f < nf; ++f) {
        if (A[f].fmt != HBK_FMT_SELL) return (int)cudaErrorInvalidValue;
        any_deferred |= v[f].deferred != 0;
        tab[f].c = make_ctx(&A[f], &v[f], &sh[f]);
        tab[f].vb0 = (unsigned)map.size();
        tab[f].nvb = group_vblocks(v[f].n, rows_per_vb);
        map.insert(map.end(), tab[f].nvb, (unsigned)f);
    }
    const unsigned nvb = (unsigned)map.size();
    if (ws_bytes < group_bytes(nf, nvb)) return (int)cudaErrorInvalidValue;
    char *base = (char *)ws;
    unsigned *bar = (unsigned *)base;
    int *err = (int *)(base + 64);
    GroupFam *dtab = (GroupFam *)(base + kGroupHead);
    unsigned *dmap = (unsigned *)(base + kGroupHead + ((sizeof(GroupFam) * (size_t)nf + 255) / 256) * 256);
    int e;
    if ((e = (int)cudaMemsetAsync(base, 0, kGroupHead, st))) return e;
    if ((e = (int)cudaMemcpyAsync(dtab, tab.data(), sizeof(GroupFam) * (size_t)nf, cudaMemcpyHostToDevice, st)))
        return e;
    if ((e = (int)cudaMemcpyAsync(dmap, map.data(), sizeof(unsigned) * (size_t)nvb, cudaMemcpyHostToDevice, st)))
        return e;
    int ctas = hbk_group_ctas(max_ctas);
    if ((unsigned)ctas > nvb) ctas = (int)nvb; /* a CTA without a virtual block would only wait at barriers */
    int withhold = g_group_withhold;
    g_group_withhold = 0;
    const GroupFam *a0 = dtab;
    const unsigned *a2 = dmap;
    void *args[] = {(void *)&a0,  (void *)&nf,  (void *)&a2,       (void *)&nvb,
                    (void *)&bar, (void *)&err, (void *)&iter_cap, (void *)&any_deferred, (void *)&withhold};
    if ((e = (int)cudaLaunchCooperativeKernel((const void *)k_group<64>, dim3(ctas), dim3(NT), args, 0, st))) return e;
    /* pageable destination: returns once the launch has finished */
    return (int)cudaMemcpyAsync(err_out, err, sizeof(int), cudaMemcpyDeviceToHost, st);
}

int hbk_loop_condition(const hbk_shifts *sh, cudaGraphConditionalHandle cond, int loop_cap, cudaStream_t st) {
    k_loop_condition<<<1, 1, 0, st>>>(sh->sc, cond, loop_cap);
    return (int)cudaGetLastError();
}

int hbk_deferred_flush(const hbk_vectors *v, const hbk_shifts *sh, int keep_p, cudaStream_t st) {
    hbk_matrix A0 = {};
    Ctx c = make_ctx(&A0, v, sh);
    const int groups = (sh->m + GROUP - 1) / GROUP;
    dim3 grid(grid_for(v->n, 1), groups);
    // x first: it reads the old Pmat, which the p pass then overwrites
    k_flush<<<grid, NT, 0, st>>>(c, keep_p, 0);
    if (keep_p) k_flush<<<grid, NT, 0, st>>>(c, keep_p, 1);
    k_flush_reset<<<grid_for(v->n, 2), NT, 0, st>>>(c, keep_p);
    return (int)cudaGetLastError();
}

int hbk_deferred_reset(const hbk_vectors *v, const hbk_shifts *sh, int keep_p, cudaStream_t st) {
    hbk_matrix A0 = {};
    Ctx c = make_ctx(&A0, v, sh);
    k_flush_reset<<<grid_for(v->n, 2), NT, 0, st>>>(c, keep_p);
    return (int)cudaGetLastError();
}

}  // extern "C"
