"""Faults made on the host, never on the GPU: a NaN in b, a NaN shift, a
shift that makes A + sigma I singular, and max_iter = 1.  Each solve must come
back (no hang) with HBICG_E_BREAKDOWN or HBICG_E_MAXITER, in the plain form
and both fused forms; a shift that breaks down records -k in conv_k and the
other shifts still reach the reference's answer.  The reference checks none
of these (src/solver_dynamic.c:166-205 divides by (r^,s), (q,y), pi and
1 - omega d unchecked) and iterates on NaN to MAX_ITER."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_BREAKDOWN, E_MAXITER = 3, 4
MODES = [dict(form="plain"), dict(form="fused", shift_mode="incremental"),
         dict(form="fused", shift_mode="deferred"), dict(form="fused", shift_mode="deferred", use_graph=False)]
IDS = ["plain", "fused-inc", "fused-def", "fused-def-eager"]


def _solve(pkg, a, b, sigma, seed, mode, max_iter=2000, tol=1e-10):
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    s = pkg.Solver(A, len(sigma), tol=tol, max_iter=max_iter, refine=False, **mode)
    res = s.run(np.asarray(b, dtype=np.float64), np.asarray(sigma, dtype=np.float64), seed=seed)
    s.close()
    A.close()
    ctx.close()
    return res


@pytest.mark.parametrize("mode", MODES, ids=IDS)
def test_nan_in_b_is_a_breakdown(cuda, pkg, mode):
    a = pkg.workloads.stencil_cd3d(8)
    b = np.full(a.n, 1.0 / np.sqrt(a.n))
    b[17] = np.nan
    res = _solve(pkg, a, b, 0.01 * np.arange(6), 0, mode)
    assert res.status == E_BREAKDOWN
    assert res.k <= 2


@pytest.mark.parametrize("mode", MODES, ids=IDS)
def test_nan_shift_stops_alone(cuda, pkg, oracle, mode):
    """Shift 2 is NaN: it breaks down at the first iteration (conv_k = -1) and
    is left out of the switch argmax; the other shifts follow the reference's
    solve of the family without it."""
    a = pkg.workloads.stencil_cd3d(8)
    b = np.full(a.n, 1.0 / np.sqrt(a.n))
    good = 0.01 * np.arange(6)
    sigma = np.insert(good, 2, np.nan)
    res = _solve(pkg, a, b, sigma, 0, mode)
    assert res.status == E_BREAKDOWN
    assert res.conv_k[2] == -1
    keep = [0, 1, 3, 4, 5, 6]
    assert np.all(res.conv_k[keep] > 0)
    want = oracle.solve(a, b, good, seed=0, tol=1e-10, max_iter=2000)
    x = np.asarray(res.x)[keep]
    err = np.max(np.abs(x - want.x)) / np.max(np.abs(want.x))
    assert err < 1e-8, err
    assert np.all(np.isfinite(np.asarray(res.x)[2]))


@pytest.mark.parametrize("mode", MODES, ids=IDS)
def test_singular_shift_returns(cuda, pkg, oracle, mode):
    """A + sigma_1 I is singular (a zero row): that system has no solution.
    The solve returns within max_iter with E_MAXITER or E_BREAKDOWN, and the
    regular shifts meet the tolerance on the true residual."""
    n = 200
    d = 1.0 + np.arange(n) / n
    a = pkg.workloads.Csr(np.arange(n + 1, dtype=np.uint32), np.arange(n, dtype=np.uint32), d.copy())
    b = np.random.default_rng(3).standard_normal(n)
    sigma = np.array([0.0, -d[0], 0.3, 0.7])
    res = _solve(pkg, a, b, sigma, 0, mode, max_iter=300)
    assert res.status in (E_BREAKDOWN, E_MAXITER)
    ok = [0, 2, 3]
    assert np.all(res.conv_k[ok] > 0)
    tr = oracle.true_residuals(a, np.asarray(res.x)[ok], b, sigma[ok])
    assert np.all(tr <= 1e-10 * 1.01), tr


@pytest.mark.parametrize("mode", MODES, ids=IDS)
def test_max_iter_one(cuda, pkg, oracle, mode):
    a = pkg.workloads.stencil_cd3d(8)
    b = np.full(a.n, 1.0 / np.sqrt(a.n))
    sigma = 0.01 * np.arange(6)
    res = _solve(pkg, a, b, sigma, 0, mode, max_iter=1)
    want = oracle.solve(a, b, sigma, seed=0, tol=1e-10, max_iter=1)
    assert res.status == E_MAXITER
    assert res.k == want.k == 2
    err = np.max(np.abs(np.asarray(res.x) - want.x)) / np.max(np.abs(want.x))
    assert err < 1e-8, err
