"""The oracle (CPU restatement of the reference's solver) pinned against the
reference: its golden vectors (tests/golden, produced by the reference's own
sources) and, where the reference sources are present, the reference itself."""
import numpy as np
import pytest

from conftest import GOLDEN, GoldenCsr, golden

SOLVER_CASES = ["stencil8_seed0", "stencil8_seed5", "stencil8_seed5_static", "stencil8_seed5_normal", "stencil2d_two_switches",
                "stencil8_maxiter5", "stencil8_single_shift", "irregular_two_switches", "irregular_fixed_seed",
                "stencil2d_seed8"]


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_restatement_matches_golden_bitwise(oracle, name):
    g = golden(name)
    a = GoldenCsr(g)
    res = oracle.solve(a, g["b"], g["sigma"], seed=int(g["seed"]), tol=float(g["tol"]),
                       max_iter=int(g["max_iter"]), switching=bool(g["switching"]), schedule=str(g["variant"]))
    assert res.k == int(g["k"])
    assert res.switches == [tuple(map(int, s)) for s in g["switches"]]
    assert np.array_equal(res.x, g["x"])
    assert np.array_equal(res.r, g["r"])


def test_golden_cases_cover_switching():
    sw = {name: len(golden(name)["switches"]) for name in SOLVER_CASES}
    assert sw["irregular_two_switches"] == 2
    assert sw["stencil8_seed5"] == 1 and sw["stencil8_seed0"] == 0
    assert int(golden("stencil8_maxiter5")["k"]) == 6  # max_iter + 1 at the limit


def test_spmv_matches_golden(oracle):
    g = golden("spmv_irregular")
    a = GoldenCsr(g)
    assert np.array_equal(oracle.spmv(a, g["x"]), g["y"])
    # the fused-multiply-add row order differs from the reference only by rounding
    y = oracle.spmv_fma(a, g["x"])
    assert np.max(np.abs(y - g["y"])) <= 1e-13 * np.max(np.abs(g["y"]))


def test_oracle_against_dense_solve(oracle, pkg):
    a = pkg.workloads.stencil_cd3d(10)
    b = np.random.default_rng(3).standard_normal(a.n)
    sigma = np.array([0.0, 0.05, 0.3, 1.0])
    res = oracle.solve(a, b, sigma, seed=0, tol=1e-13, max_iter=2000)
    dense = a.to_dense()
    for j, s in enumerate(sigma):
        xd = np.linalg.solve(dense + s * np.eye(a.n), b)
        assert np.max(np.abs(res.x[j] - xd)) <= 1e-9 * np.max(np.abs(xd))


def test_manufactured_solution_seed_system(oracle, pkg):
    # x* = 1 and b = (A + sigma_seed I) 1 (the reference's archived driver idea)
    a = pkg.workloads.stencil_cd3d(12)
    sigma = np.array([0.02, 0.1, 0.5])
    b = a.matvec(np.ones(a.n)) + sigma[0]
    res = oracle.solve(a, b, sigma, seed=0, tol=1e-13, max_iter=2000)
    assert np.max(np.abs(res.x[0] - 1.0)) < 1e-9


def test_true_residual_meets_tolerance_c1(oracle, pkg):
    f = pkg.workloads.family("c1")
    res = oracle.solve(f.a, f.b, f.sigma, seed=0, tol=f.tol, max_iter=f.max_iter)
    assert res.k == 81
    tr = oracle.true_residuals(f.a, res.x, f.b, f.sigma)
    assert tr.max() <= f.tol * (1 + 1e-3)


ref_only = pytest.mark.skipif("not __import__('oracle').ref_available()", reason="reference sources absent")


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference build (oracle/_ref) not present")
    return oracle


@pytest.mark.parametrize("seed", [0, 7, 15])
@pytest.mark.parametrize("variant", ["dynamic", "static", "normal"])
def test_restatement_matches_reference_c1(ref, pkg, seed, variant):
    f = pkg.workloads.family("c1")
    want = ref.ref_solve(f.a, f.b, f.sigma, seed=seed, tol=f.tol, max_iter=f.max_iter, variant=variant)
    got = ref.solve(f.a, f.b, f.sigma, seed=seed, tol=f.tol, max_iter=f.max_iter, schedule=variant)
    assert got.k == want.k and got.switches == want.switches
    assert np.array_equal(got.x, want.x) and np.array_equal(got.r, want.r)


@pytest.mark.parametrize("trial", range(4))
def test_restatement_matches_reference_random(ref, pkg, trial):
    rng = np.random.default_rng(100 + trial)
    a = pkg.workloads.irregular_powerlaw(int(rng.integers(200, 900)), mean_len=9, max_len=80, seed=trial)
    m = int(rng.integers(1, 9))
    sigma = rng.uniform(-0.1, 1.0, m)
    b = rng.standard_normal(a.n)
    seed = int(rng.integers(0, m))
    for switching in (True, False):
        want = ref.ref_solve(a, b, sigma, seed=seed, tol=1e-10, max_iter=600, switching=switching)
        got = ref.solve(a, b, sigma, seed=seed, tol=1e-10, max_iter=600, switching=switching)
        assert got.k == want.k and got.switches == want.switches
        assert np.array_equal(got.x, want.x)


def test_spmv_matches_reference(ref, pkg):
    a = pkg.workloads.irregular_powerlaw(5000, seed=4)
    x = np.random.default_rng(5).standard_normal(a.n)
    assert np.array_equal(ref.spmv(a, x), ref.ref_spmv(a, x))


def test_golden_files_present():
    names = {p.name for p in GOLDEN.iterdir()}
    for n in SOLVER_CASES + ["spmv_irregular", "mm_loader"]:
        assert f"{n}.npz" in names
