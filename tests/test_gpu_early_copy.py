"""Deferred mode into pinned host memory: the solutions of shifts that have
converged by a basis flush are copied to the caller's buffer during the solve
(a second stream).  The result must be the same, bit for bit, as with a
pageable buffer, which is copied once at the end."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pinned_output_matches_pageable(cuda, pkg):
    torch = cuda
    f = pkg.workloads.family("c1", scale=16)
    m = len(f.sigma)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, f.a.ptr, f.a.col, f.a.val)
    s = pkg.Solver(A, m, tol=f.tol, max_iter=f.max_iter, shift_mode="deferred", basis_block=6, refine=False)
    x_pageable = np.zeros((m, f.a.n))
    res = s.run(f.b, f.sigma, seed=f.seed, x=x_pageable)
    assert res.shift_mode == "deferred" and res.flushes >= 3
    assert len(set(res.conv_k.tolist())) > 2  # shifts finish at different flushes
    x_pinned = torch.full((m, f.a.n), np.nan, dtype=torch.float64).pin_memory()
    res2 = s.run(f.b, f.sigma, seed=f.seed, x=x_pinned.numpy())
    assert res2.k == res.k
    assert np.array_equal(x_pinned.numpy(), x_pageable)
    s.close()
    A.close()
    ctx.close()


def test_pinned_output_with_refine(cuda, pkg):
    torch = cuda
    f = pkg.workloads.family("c1", scale=16)
    m = len(f.sigma)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, f.a.ptr, f.a.col, f.a.val)
    s = pkg.Solver(A, m, tol=f.tol, max_iter=f.max_iter, shift_mode="deferred", basis_block=6, refine=True,
                   true_residuals=True)
    x_pageable = np.zeros((m, f.a.n))
    res = s.run(f.b, f.sigma, seed=f.seed, x=x_pageable)
    x_pinned = torch.zeros((m, f.a.n), dtype=torch.float64).pin_memory()
    res2 = s.run(f.b, f.sigma, seed=f.seed, x=x_pinned.numpy())
    assert res2.refined == res.refined
    assert np.array_equal(x_pinned.numpy(), x_pageable)
    assert res2.max_true_residual <= f.tol * (1 + 1e-3)
    s.close()
    A.close()
    ctx.close()


def test_dropin_pinned_matches_pageable(cuda, pkg):
    torch = cuda
    f = pkg.workloads.family("c2", scale=40)  # deferred mode (n m >= 2^21) in the drop-in call
    m, n = len(f.sigma), f.a.n
    outs = []
    for pinned in (False, True):
        x = torch.zeros((m, n), dtype=torch.float64)
        r = torch.from_numpy(f.b.copy())
        if pinned:
            x, r = x.pin_memory(), r.pin_memory()
        k = pkg.dropin_raw("dynamic", torch.from_numpy(f.a.ptr), torch.from_numpy(f.a.col), torch.from_numpy(f.a.val),
                           x, r, torch.from_numpy(f.sigma), f.seed, f.tol, f.max_iter)
        outs.append((k, x.numpy().copy(), r.numpy().copy()))
    assert outs[0][0] == outs[1][0]
    assert np.array_equal(outs[0][1], outs[1][1]) and np.array_equal(outs[0][2], outs[1][2])
