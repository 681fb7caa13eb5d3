"""hbicg_true_residuals_noalloc: the residual check for callers that cannot
call cudaMalloc (another component owns the device memory, or the caller is in
a loop or callback where an allocation is not allowed).  It must give the same
true relative residuals as the solver's own check (hbicg_solver_run with
true_residuals on), call after call, while taking its scratch from the
library's static device array.  Collected last on purpose: it shares no state
with the other tests and must pass alone or after them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _family(pkg, side, m, seed):
    a = pkg.workloads.stencil_cd3d(side, side + 1, side + 2)  # odd n: x rows are not 32-aligned
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(a.n)
    sigma = np.sort(rng.uniform(1e-3, 1.0, m))
    return a, b, sigma


@pytest.mark.parametrize("side,m", [(9, 5), (21, 64)])
def test_noalloc_matches_solver_check_twice(cuda, pkg, side, m):
    torch = cuda
    a, b_h, sig_h = _family(pkg, side, m, side)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    s = pkg.Solver(A, m, tol=1e-10, max_iter=2000, true_residuals=True)
    b = torch.tensor(b_h, device="cuda")
    sig = torch.tensor(sig_h, device="cuda")
    x = torch.zeros((m, a.n), dtype=torch.float64, device="cuda")
    ref = s.run(b, sig, seed=0, x=x)
    torch.cuda.synchronize()
    want = ref.true_residual
    assert want is not None and np.all(want > 0) and np.all(want < 2e-10)
    stream = torch.cuda.Stream()
    for _ in range(2):
        res = torch.full((m,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        pkg.true_residuals_noalloc(A, x, b, sig, res, stream=stream.cuda_stream)
        stream.synchronize()
        got = res.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
    s.close()
    A.close()
    ctx.close()


def test_noalloc_rejects_too_many_shifts(cuda, pkg):
    torch = cuda
    a, b_h, _ = _family(pkg, 5, 1, 0)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    m = 65
    x = torch.zeros((m, a.n), dtype=torch.float64, device="cuda")
    b = torch.tensor(b_h, device="cuda")
    sig = torch.zeros(m, dtype=torch.float64, device="cuda")
    res = torch.zeros(m, dtype=torch.float64, device="cuda")
    with pytest.raises(pkg.HbicgError, match="64"):
        pkg.true_residuals_noalloc(A, x, b, sig, res)
    A.close()
    ctx.close()
