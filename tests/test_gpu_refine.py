"""params.refine: the true residual of every shift is checked after the solve
and shifts above tol are corrected through the residual equation.  On two
families of config 4 the recursive residual converges while the true one ends
above tol (1e-10); with refine every shift meets it.  A solve that needs no
correction is unchanged bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("index", [34, 63])
def test_refine_brings_true_residual_to_tol(cuda, pkg, index):
    f = pkg.workloads.batched_families(256)[index]
    kw = dict(seed=f.seed, tol=1e-10, max_iter=10000, true_residuals=True)
    plain = pkg.solve(f.a, f.b, f.sigma, refine=False, **kw)
    ref = pkg.solve(f.a, f.b, f.sigma, refine=True, **kw)
    assert ref.max_true_residual <= 1e-10
    if plain.max_true_residual > 1e-10:
        assert ref.refined >= 1
    assert ref.k == plain.k  # the main solve is the same


def test_refine_without_need_changes_nothing(cuda, pkg):
    a = pkg.workloads.stencil_cd3d(10)
    b = np.full(a.n, 1.0 / np.sqrt(a.n))
    sigma = 0.01 * np.arange(8, dtype=np.float64)
    kw = dict(seed=0, tol=1e-10, max_iter=2000, true_residuals=True)
    r0 = pkg.solve(a, b, sigma, refine=False, **kw)
    r1 = pkg.solve(a, b, sigma, refine=True, **kw)
    assert r0.max_true_residual <= 1e-10
    assert r1.refined == 0 and np.array_equal(r0.x, r1.x)
