"""Solver parity on the GPU against the oracle and the reference's golden
vectors.  Tolerances (FP64): solutions within 1e-8 relative to max|x| of the
reference's answers; iteration counts within 2% (at least one iteration) of
the oracle's envelope; seed-switch sequences identical to one the oracle
produces; every shift's true relative residual within the tolerance (1e-3
relative slack: the test is on the recursive residual, as in the reference).

The envelope: the oracle is run on the same inputs and on b perturbed by
1e-14 relative noise.  Where a shift's recursive residual crosses the
tolerance within rounding of the threshold, or two residual factors tie in the
seed-switch argmax, those runs differ (C1 with seed 15 ends at k = 81 or 84
depending on the last bits of b); a GPU result is accepted when it lies within
what the reference's own arithmetic produces under such perturbations."""
from functools import lru_cache
import numpy as np
import pytest

from conftest import GoldenCsr, golden

pytestmark = pytest.mark.gpu

X_RTOL = 1e-8
MODES = [
    dict(form="plain"),
    dict(form="fused", shift_mode="incremental"),
    dict(form="fused", shift_mode="deferred"),
    dict(form="fused", shift_mode="incremental", use_graph=False),
    dict(form="fused", shift_mode="deferred", use_graph=False),
    dict(form="fused", shift_mode="incremental", use_graph="persistent"),
    dict(form="fused", shift_mode="deferred", use_graph="persistent"),
]
MODE_IDS = ["plain", "fused-inc", "fused-def", "fused-inc-eager", "fused-def-eager", "fused-inc-persistent",
            "fused-def-persistent"]


def k_close(k, want):
    return abs(k - want) <= max(1, int(0.02 * want))


def envelope(oracle, a, b, sigma, seed, tol, max_iter, switching=True, runs=6, want=None):
    """(k_lo, k_hi, switch sequences, conv_k lo, conv_k hi) over perturbed oracle runs"""
    outs = [want] if want is not None else []
    for t in range(runs):
        bb = b if t == 0 else b * (1 + 1e-14 * np.random.default_rng(t).standard_normal(b.shape[0]))
        outs.append(oracle.solve(a, bb, sigma, seed=seed, tol=tol, max_iter=max_iter, switching=switching))
    ks = [o.k for o in outs]
    conv = np.array([o.conv_k for o in outs if o.conv_k is not None])
    return min(ks), max(ks), {tuple(o.switches) for o in outs}, conv.min(axis=0), conv.max(axis=0)


def check_envelope(res, env):
    lo, hi, sws, clo, chi = env
    assert lo - max(1, int(0.02 * lo)) <= res.k <= hi + max(1, int(0.02 * hi)), (res.k, lo, hi)
    assert tuple(res.switches) in sws, (res.switches, sws)
    assert np.all(res.conv_k >= clo - 1) and np.all(res.conv_k <= chi + 1), (res.conv_k, clo, chi)


def x_err(x, want):
    return np.max(np.abs(x - want)) / max(np.max(np.abs(want)), 1e-300)


GOLDEN_CASES = ["stencil8_seed0", "stencil8_seed5", "stencil8_maxiter5", "stencil8_single_shift",
                "stencil2d_two_switches", "stencil2d_seed8"]
# Near-indefinite shifts (sigma = -0.058 and -0.065 on a power-law matrix): the
# iteration at which these systems converge, and hence where the seed switches,
# moves by tens of iterations under 1e-14 relative perturbations of b in the
# oracle itself.  The solutions still agree; iteration counts within 10%.
CHAOTIC_CASES = ["irregular_two_switches", "irregular_fixed_seed"]


@lru_cache(maxsize=None)
def golden_envelope(name):
    import __graft_entry__ as graft

    g = golden(name)
    return envelope(graft.load_oracle(), GoldenCsr(g), g["b"], g["sigma"], int(g["seed"]), float(g["tol"]),
                    int(g["max_iter"]), bool(g["switching"]))


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden(cuda, pkg, name, mode):
    g = golden(name)
    a = GoldenCsr(g)
    res = pkg.solve(a, g["b"], g["sigma"], seed=int(g["seed"]), tol=float(g["tol"]), max_iter=int(g["max_iter"]),
                    switching=bool(g["switching"]), **mode)
    assert k_close(res.k, int(g["k"])), (res.k, int(g["k"]))
    assert res.switches == [tuple(map(int, s)) for s in g["switches"]]
    if name == "stencil8_maxiter5":
        assert res.k == 6
    assert x_err(res.x, g["x"]) < X_RTOL
    check_envelope(res, golden_envelope(name))


@pytest.mark.parametrize("mode", MODES[:3], ids=MODE_IDS[:3])
@pytest.mark.parametrize("name", CHAOTIC_CASES)
def test_golden_near_ties(cuda, pkg, name, mode):
    g = golden(name)
    res = pkg.solve(GoldenCsr(g), g["b"], g["sigma"], seed=int(g["seed"]), tol=float(g["tol"]),
                    max_iter=int(g["max_iter"]), switching=bool(g["switching"]), true_residuals=True, **mode)
    lo, hi, _, _, _ = golden_envelope(name)
    assert min(lo, int(g["k"])) * 0.9 <= res.k <= max(hi, int(g["k"])) * 1.1
    assert np.all(res.conv_k > 0)
    assert x_err(res.x, g["x"]) < X_RTOL
    assert res.max_true_residual <= float(g["tol"]) * 1.05


@lru_cache(maxsize=None)
def c1_envelope(seed):
    import __graft_entry__ as graft

    f = graft.load_package().workloads.family("c1")
    return envelope(graft.load_oracle(), f.a, f.b, f.sigma, seed, f.tol, f.max_iter)


@pytest.mark.parametrize("seed", [0, 15])
@pytest.mark.parametrize("mode", MODES[:3] + MODES[5:], ids=MODE_IDS[:3] + MODE_IDS[5:])
def test_c1_full(cuda, pkg, oracle, seed, mode):
    f = pkg.workloads.family("c1")
    want = oracle.solve(f.a, f.b, f.sigma, seed=seed, tol=f.tol, max_iter=f.max_iter)
    res = pkg.solve(f.a, f.b, f.sigma, seed=seed, tol=f.tol, max_iter=f.max_iter, true_residuals=True, **mode)
    check_envelope(res, c1_envelope(seed))
    assert x_err(res.x, want.x) < X_RTOL
    assert res.max_true_residual <= f.tol * (1 + 1e-3)
    tr = oracle.true_residuals(f.a, res.x, f.b, f.sigma)
    assert np.allclose(tr, res.true_residual, rtol=1e-4, atol=1e-16)


def test_dense_direct_solve(cuda, pkg):
    a = pkg.workloads.stencil_cd3d(16)
    b = np.random.default_rng(11).standard_normal(a.n)
    sigma = np.array([1e-3, 0.01, 0.1, 0.5, 1.0])
    res = pkg.solve(a, b, sigma, seed=0, tol=1e-13, max_iter=3000)
    dense = a.to_dense()
    for j, s in enumerate(sigma):
        xd = np.linalg.solve(dense + s * np.eye(a.n), b)
        assert x_err(res.x[j], xd) < 1e-9


@pytest.mark.parametrize("variant", ["dynamic", "static", "normal"])
def test_dropin_entry_points(cuda, pkg, oracle, variant):
    g = golden("stencil8_seed5")
    a = GoldenCsr(g)
    k, x, r = pkg.dropin_solve(variant, a, g["b"], g["sigma"], seed=5, tol=1e-10, max_iter=10000)
    assert k_close(k, int(g["k"]))
    assert x_err(x, g["x"]) < X_RTOL
    bn = np.linalg.norm(g["b"])
    assert np.linalg.norm(r - g["r"]) / bn < 1e-9  # final seed residual, overwritten like r_loc


def test_dropin_defaults_are_reference_constants(cuda, pkg, oracle):
    f = pkg.workloads.family("c1", scale=10)
    k, x, _ = pkg.dropin_solve("dynamic", f.a, f.b, f.sigma[:4], seed=0)  # EPS 1e-12, MAX_ITER 2000
    want = oracle.solve(f.a, f.b, f.sigma[:4], seed=0, tol=1e-12, max_iter=2000)
    assert k_close(k, want.k) and x_err(x, want.x) < X_RTOL


def test_zero_rhs(cuda, pkg):
    a = pkg.workloads.stencil_cd3d(6)
    res = pkg.solve(a, np.zeros(a.n), np.array([0.0, 0.5]), seed=0, tol=1e-10, max_iter=100)
    assert res.k == 1 and np.all(res.x == 0.0) and res.status == 0


@pytest.mark.parametrize("mode", ["incremental", "deferred"])
def test_fixed_seed_matches_reference_fixed_seed(cuda, pkg, mode):
    g = golden("irregular_fixed_seed")
    res = pkg.solve(GoldenCsr(g), g["b"], g["sigma"], seed=int(g["seed"]), tol=1e-10, max_iter=3000,
                    switching=False, shift_mode=mode)
    lo, hi, _, _, _ = golden_envelope("irregular_fixed_seed")
    assert min(lo, int(g["k"])) * 0.9 <= res.k <= max(hi, int(g["k"])) * 1.1 and res.switches == []
    assert x_err(res.x, g["x"]) < X_RTOL


def test_deferred_basis_flushes(cuda, pkg, oracle):
    f = pkg.workloads.family("c1", scale=20)
    want = oracle.solve(f.a, f.b, f.sigma, seed=15, tol=f.tol, max_iter=f.max_iter)
    # a basis of a few dozen slots forces several flushes during the solve
    res = pkg.solve(f.a, f.b, f.sigma, seed=15, tol=f.tol, max_iter=f.max_iter, shift_mode="deferred",
                    basis_mem_frac=1e-5, true_residuals=True)
    assert res.flushes >= 1
    check_envelope(res, envelope(oracle, f.a, f.b, f.sigma, 15, f.tol, f.max_iter))
    assert x_err(res.x, want.x) < X_RTOL
    assert res.max_true_residual <= f.tol * (1 + 1e-3)


def test_solver_reuse_device_pointers(cuda, pkg, oracle):
    torch = cuda
    f = pkg.workloads.family("c1", scale=12)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, f.a.ptr, f.a.col, f.a.val)
    s = pkg.Solver(A, len(f.sigma), tol=f.tol, max_iter=f.max_iter)
    want = oracle.solve(f.a, f.b, f.sigma, seed=3, tol=f.tol, max_iter=f.max_iter)
    env = envelope(oracle, f.a, f.b, f.sigma, 3, f.tol, f.max_iter)
    b = torch.tensor(f.b, device="cuda")
    sig = torch.tensor(f.sigma, device="cuda")
    x = torch.zeros((len(f.sigma), f.a.n), dtype=torch.float64, device="cuda")
    for _ in range(2):  # graphs are captured once and replayed
        res = s.run(b, sig, seed=3, x=x)
        torch.cuda.synchronize()
        check_envelope(res, env)
        assert x_err(x.cpu().numpy(), want.x) < X_RTOL
    s.close()
    A.close()
    ctx.close()


@pytest.mark.parametrize("shift_mode", ["incremental", "deferred"])
@pytest.mark.parametrize("name", ["stencil2d_two_switches", "stencil8_maxiter5", "stencil2d_seed8"])
def test_loop_graph_equals_chunked_graph(cuda, pkg, name, shift_mode):
    """The iterations as one conditional while node in a CUDA graph
    (use_graph="loop") and as replayed chunks of iterations (the default) run
    the same kernels in the same order: identical k, switches, convergence
    iterations and bits of x; and both end at the reference's answer."""
    g = golden(name)
    kw = dict(seed=int(g["seed"]), tol=float(g["tol"]), max_iter=int(g["max_iter"]), switching=bool(g["switching"]),
              shift_mode=shift_mode, refine=False)
    loop = pkg.solve(GoldenCsr(g), g["b"], g["sigma"], use_graph="loop", **kw)
    chunk = pkg.solve(GoldenCsr(g), g["b"], g["sigma"], **kw)
    assert loop.k == chunk.k and loop.switches == chunk.switches
    assert np.array_equal(loop.conv_k, chunk.conv_k)
    assert np.array_equal(loop.x, chunk.x)
    assert x_err(loop.x, g["x"]) < X_RTOL
