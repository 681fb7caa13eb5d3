"""Tensor-core basis flush (tcgen05, BF16 digit products) against an
extended-precision reference: every output within a few FP64 units in the
last place of the size of its terms, i.e. as accurate as an FP64 product."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_tc(pkg, torch, V, Xc, Pc, own, X, Pm, n, L, m, keep_p):
    lib = pkg.lib()
    fn = lib.hbk_flush_tc_run
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_uint, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbk_flush_tc_workspace_bytes.restype = C.c_size_t
    lib.hbk_flush_tc_workspace_bytes.argtypes = [C.c_int]
    ws = torch.zeros(int(lib.hbk_flush_tc_workspace_bytes(m)) // 8 + 1, dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ld = V.stride(0)
    cap = Xc.stride(0)
    rc = fn(V.data_ptr(), ld, n, L, Xc.data_ptr(), Pc.data_ptr(), cap, own.data_ptr(), m, X.data_ptr(),
            Pm.data_ptr() if Pm is not None else None, keep_p, ws.data_ptr(), err.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0
    assert int(err.item()) == 0
    return X, Pm


def _case(m, L, n, seed, zero_cols=False):
    rng = np.random.default_rng(seed)
    ld = (n + 31) // 32 * 32
    V = np.zeros((L, ld))
    scale = 10.0 ** (-rng.uniform(0, 8, L))  # slots of very different size, as residuals shrink
    V[:, :n] = rng.standard_normal((L, n)) * scale[:, None]
    V[:, : n // 7] *= 1e-3  # uneven magnitudes along each vector too
    if zero_cols:
        V[:, 5:9] = 0.0
    V[rng.integers(0, L, 3), :] = 0.0  # unused slots
    cap = L + 5
    Xc = np.zeros((m, cap))
    Pc = np.zeros((m, cap))
    Xc[:, :L] = rng.standard_normal((m, L)) / scale[None, :] * 10.0 ** rng.uniform(-2, 2, (m, 1))
    Pc[:, :L] = rng.standard_normal((m, L)) / scale[None, :]
    own = rng.standard_normal((m, 2))
    X = np.zeros((m, ld))
    Pm = np.zeros((m, ld))
    X[:, :n] = rng.standard_normal((m, n)) * 10.0
    Pm[:, :n] = rng.standard_normal((m, n))
    return V, Xc, Pc, own, X, Pm, ld


def _reference(V, Xc, Pc, own, X, Pm, n, L):
    ext = np.longdouble
    Vn = V[:L, :n].astype(ext)
    gx = Xc[:, :L].astype(ext) @ Vn
    gp = Pc[:, :L].astype(ext) @ Vn
    x = X[:, :n].astype(ext) + own[:, :1].astype(ext) * Pm[:, :n].astype(ext) + gx
    p = own[:, 1:2].astype(ext) * Pm[:, :n].astype(ext) + gp
    sx = np.abs(X[:, :n]) + np.abs(own[:, :1] * Pm[:, :n]) + np.abs(Xc[:, :L]) @ np.abs(V[:L, :n])
    sp = np.abs(own[:, 1:2] * Pm[:, :n]) + np.abs(Pc[:, :L]) @ np.abs(V[:L, :n])
    return x, p, sx, sp


@pytest.mark.parametrize("m,L,n,keep_p", [(64, 51, 5003, 1), (5, 17, 1000, 1), (70, 64, 777, 1), (64, 51, 4801, 0)])
def test_tc_flush_matches_extended_precision(cuda, pkg, m, L, n, keep_p):
    torch = cuda
    V, Xc, Pc, own, X, Pm, ld = _case(m, L, n, seed=m * 7 + L, zero_cols=(m == 5))
    x_ref, p_ref, sx, sp = _reference(V, Xc, Pc, own, X, Pm, n, L)
    tV = torch.tensor(V, device="cuda")
    tX = torch.tensor(X, device="cuda")
    tPm = torch.tensor(Pm, device="cuda")
    _run_tc(pkg, torch, tV, torch.tensor(Xc, device="cuda"), torch.tensor(Pc, device="cuda"),
            torch.tensor(own, device="cuda"), tX, tPm, n, L, m, keep_p)
    ulp = 2.0 ** -52
    x = tX.cpu().numpy()[:, :n]
    err_x = np.abs(x.astype(np.longdouble) - x_ref).astype(np.float64)
    assert np.all(err_x <= 4 * ulp * sx + 1e-300), float(np.max(err_x / (sx + 1e-300)))
    pm = tPm.cpu().numpy()[:, :n]
    if keep_p:
        err_p = np.abs(pm.astype(np.longdouble) - p_ref).astype(np.float64)
        assert np.all(err_p <= 4 * ulp * sp + 1e-300), float(np.max(err_p / (sp + 1e-300)))
    else:
        assert np.array_equal(pm, Pm[:, :n])
    # columns past n untouched
    assert np.array_equal(tX.cpu().numpy()[:, n:], X[:, n:])


def test_tc_flush_in_solver_matches_fp64_flush(cuda, pkg, oracle):
    f = pkg.workloads.family("c1", scale=20)
    kw = dict(seed=15, tol=f.tol, max_iter=f.max_iter, shift_mode="deferred", basis_block=8, true_residuals=True)
    a = pkg.solve(f.a, f.b, f.sigma, flush="fp64", **kw)
    b = pkg.solve(f.a, f.b, f.sigma, flush="tensor", **kw)
    assert a.flushes >= 3 and b.flushes == a.flushes
    assert b.k == a.k and b.switches == a.switches
    assert np.max(np.abs(b.x - a.x)) <= 1e-12 * np.max(np.abs(a.x))
    assert b.max_true_residual <= f.tol * (1 + 1e-3)
