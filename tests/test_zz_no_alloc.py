"""hbicg_true_residuals_noalloc: the residual check for callers that cannot
call cudaMalloc (another component owns the device memory, or the caller is in
a loop or callback where an allocation is not allowed).  It must give the same
true relative residuals as the solver's own check (hbicg_solver_run with
true_residuals on), call after call, while taking its scratch from the
library's static device array, and agree with an independent FP64 residual
computed on the host by the oracle.  Collected last on purpose: it shares no
state with the other tests and must pass alone or after them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
# against the oracle's host residual: both are FP64, summed in different orders
# (fused multiply-adds on the GPU, separate products and sums on the host); the
# residual is ~1e-10 of ||b||, so rounding of A x at ~1e-16 moves it by ~1e-6
RTOL_ORACLE = 1e-4


def _family(pkg, side, m, seed):
    a = pkg.workloads.stencil_cd3d(side, side + 1, side + 2)  # odd n: x rows are not 32-aligned
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(a.n)
    sigma = np.sort(rng.uniform(1e-3, 1.0, m))
    return a, b, sigma


@pytest.mark.parametrize("side,m", [(9, 5), (21, 64)])
def test_noalloc_matches_solver_check_twice(cuda, pkg, oracle, side, m):
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
    host = oracle.true_residuals(a, x.cpu().numpy(), b_h, sig_h)
    stream = torch.cuda.Stream()
    for _ in range(2):
        res = torch.full((m,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        pkg.true_residuals_noalloc(A, x, b, sig, res, stream=stream.cuda_stream)
        stream.synchronize()
        got = res.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
        np.testing.assert_allclose(got, host, rtol=RTOL_ORACLE, atol=0)
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
