"""Tensor-core basis flush (tcgen05, BF16 digit products) against an
extended-precision reference: every output within a few FP64 units in the
last place of the size of its terms, i.e. as accurate as an FP64 product."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


PANEL = 48


def _to_panels(A, n, fill=None):
    """Row-major (m, >= n) -> flat panel-major array: element i of row j at
    ((i // 48) m + j) 48 + i % 48; the tail of the last panel is `fill`."""
    m = A.shape[0]
    npn = -(-n // PANEL)
    pad = np.full((m, npn * PANEL), np.nan if fill is None else fill)
    pad[:, :n] = A[:, :n]
    return np.ascontiguousarray(pad.reshape(m, npn, PANEL).transpose(1, 0, 2)).reshape(-1)


def _from_panels(flat, m, n):
    npn = -(-n // PANEL)
    full = flat.reshape(npn, m, PANEL).transpose(1, 0, 2).reshape(m, npn * PANEL)
    return full[:, :n], full[:, n:]


def _run_tc(pkg, torch, V, Xc, Pc, own, X, Pm, n, L, m, keep_p, conv_k=None, k_last=0):
    """X, Pm: row-major numpy arrays; they go to the kernel panel-major (tail
    of the last panel = 7.0) and come back row-major with that tail."""
    lib = pkg.lib()
    fn = lib.hbk_flush_tc_run_live
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_uint, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p]
    lib.hbk_flush_tc_workspace_bytes.restype = C.c_size_t
    lib.hbk_flush_tc_workspace_bytes.argtypes = [C.c_int]
    ws = torch.zeros(int(lib.hbk_flush_tc_workspace_bytes(m)) // 8 + 1, dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ck = torch.tensor(conv_k, dtype=torch.int32, device="cuda") if conv_k is not None else None
    tX = torch.tensor(_to_panels(X, n, 7.0), device="cuda")
    tP = torch.tensor(_to_panels(Pm, n, 7.0), device="cuda") if Pm is not None else None
    ld = V.stride(0)
    cap = Xc.stride(0)
    rc = fn(V.data_ptr(), ld, n, L, Xc.data_ptr(), Pc.data_ptr(), cap, own.data_ptr(), m, tX.data_ptr(),
            tP.data_ptr() if tP is not None else None, keep_p, ck.data_ptr() if ck is not None else None, k_last,
            None, ws.data_ptr(), err.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0
    assert int(err.item()) == 0
    x, xt = _from_panels(tX.cpu().numpy(), m, n)
    p, pt = (None, None) if tP is None else _from_panels(tP.cpu().numpy(), m, n)
    return x, p, xt, pt


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


# (20, 40, 29213): 609 tiles, so every CTA runs 4 or 5 tiles and both basis-digit
# buffers are reused; two TMEM quadrants live; a partial last panel
@pytest.mark.parametrize("m,L,n,keep_p", [(64, 51, 5003, 1), (5, 17, 1000, 1), (70, 64, 777, 1), (64, 51, 4801, 0),
                                          (20, 40, 29213, 1)])
def test_tc_flush_matches_extended_precision(cuda, pkg, m, L, n, keep_p):
    torch = cuda
    V, Xc, Pc, own, X, Pm, ld = _case(m, L, n, seed=m * 7 + L, zero_cols=(m == 5))
    x_ref, p_ref, sx, sp = _reference(V, Xc, Pc, own, X, Pm, n, L)
    x, pm, xt, pt = _run_tc(pkg, torch, torch.tensor(V, device="cuda"), torch.tensor(Xc, device="cuda"),
                            torch.tensor(Pc, device="cuda"), torch.tensor(own, device="cuda"), X, Pm, n, L, m, keep_p)
    ulp = 2.0 ** -52
    err_x = np.abs(x.astype(np.longdouble) - x_ref).astype(np.float64)
    assert np.all(err_x <= 4 * ulp * sx + 1e-300), float(np.max(err_x / (sx + 1e-300)))
    if keep_p:
        err_p = np.abs(pm.astype(np.longdouble) - p_ref).astype(np.float64)
        assert np.all(err_p <= 4 * ulp * sp + 1e-300), float(np.max(err_p / (sp + 1e-300)))
    else:
        assert np.array_equal(pm, Pm[:, :n])
    # the tail of the last panel (elements past n) untouched
    assert np.all(xt == 7.0) and np.all(pt == 7.0)


def test_tc_flush_in_solver_matches_fp64_flush(cuda, pkg, oracle):
    f = pkg.workloads.family("c1", scale=20)
    kw = dict(seed=15, tol=f.tol, max_iter=f.max_iter, shift_mode="deferred", basis_block=8, true_residuals=True)
    a = pkg.solve(f.a, f.b, f.sigma, flush="fp64", **kw)
    b = pkg.solve(f.a, f.b, f.sigma, flush="tensor", **kw)
    assert a.flushes >= 3 and b.flushes == a.flushes
    assert b.k == a.k and b.switches == a.switches
    assert np.max(np.abs(b.x - a.x)) <= 1e-12 * np.max(np.abs(a.x))
    assert b.max_true_residual <= f.tol * (1 + 1e-3)


@pytest.mark.parametrize("m,n,pattern", [(64, 5003, "every3"), (70, 2401, "two_groups"), (64, 1000, "seventeen"),
                                         (40, 777, "none")])
def test_tc_flush_live_shifts_only(cuda, pkg, m, n, pattern):
    """Shifts that converged by the previous flush (0 < conv_k <= k_last) keep
    their rows bit for bit, whatever their coefficients; the others are formed
    as in the all-live flush."""
    torch = cuda
    L, k_last = 51, 100
    V, Xc, Pc, own, X, Pm, ld = _case(m, L, n, seed=m + n)
    rng = np.random.default_rng(m)
    conv = np.zeros(m, dtype=np.int32)
    if pattern == "every3":
        conv[::3] = rng.integers(1, k_last + 1, len(conv[::3]))  # dead
        conv[1::3] = k_last + 1 + rng.integers(0, 20, len(conv[1::3]))  # converged in this block: live
    elif pattern == "two_groups":
        conv[:] = rng.integers(1, k_last + 1, m)
        conv[[0, 5, 9, 33, 63, 64, 69]] = 0  # live shifts at both ends of both groups
    elif pattern == "seventeen":
        conv[:] = 7
        conv[rng.choice(m, 17, replace=False)] = 0
    else:
        conv[:] = k_last  # converged at the last iteration the previous flush covered: dead
    dead = (conv > 0) & (conv <= k_last)
    x_ref, p_ref, sx, sp = _reference(V, Xc, Pc, own, X, Pm, n, L)
    x, pm, xt, pt = _run_tc(pkg, torch, torch.tensor(V, device="cuda"), torch.tensor(Xc, device="cuda"),
                            torch.tensor(Pc, device="cuda"), torch.tensor(own, device="cuda"), X, Pm, n, L, m, 1,
                            conv_k=conv, k_last=k_last)
    assert np.array_equal(x[dead], X[dead, :n]) and np.array_equal(pm[dead], Pm[dead, :n])
    ulp = 2.0 ** -52
    lv = ~dead
    if lv.any():
        err_x = np.abs(x[lv].astype(np.longdouble) - x_ref[lv]).astype(np.float64)
        assert np.all(err_x <= 4 * ulp * sx[lv] + 1e-300)
        err_p = np.abs(pm[lv].astype(np.longdouble) - p_ref[lv]).astype(np.float64)
        assert np.all(err_p <= 4 * ulp * sp[lv] + 1e-300)
    assert np.all(xt == 7.0) and np.all(pt == 7.0)
