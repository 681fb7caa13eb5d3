"""torch.autograd binding of the shifted family solve.

    X = shifted_solve(ptr, col, val, b, sigma)      # X[j] = (A + sigma_j I)^{-1} b

is differentiable in `val` (A's values on its fixed pattern), `b` and
`sigma`.  Backward, for an upstream gradient G = dL/dX, solves the transposed
systems (A^T + sigma_j I) lam_j = G_j and returns
    dL/dval[e] = -sum_j lam_j[row e] x_j[col e],  dL/db = sum_j lam_j,
    dL/dsigma_j = -lam_j . x_j.
When the rows of G are all multiples of one vector (as for a loss
sum_j w_j c^T x_j), the transposed systems are one shifted family with
right-hand side c (one solve); otherwise each shift is solved on its own.
The reference has no adjoint; the forward solve is the reference's algorithm.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Context, Matrix, Solver

_RANK1_TOL = 1e-13


def _rank_one(G: torch.Tensor):
    """(w, g) with G = w[:, None] * g[None, :] to rounding, else None."""
    norms = torch.linalg.vector_norm(G, dim=1)
    k = int(torch.argmax(norms))
    g = G[k]
    gg = float(g @ g)
    if gg == 0.0:
        return torch.zeros(G.shape[0], dtype=G.dtype, device=G.device), g
    w = (G @ g) / gg
    err = float(torch.max(torch.abs(G - w[:, None] * g[None, :])))
    if err <= _RANK1_TOL * float(torch.max(torch.abs(G))):
        return w, g
    return None


class _ShiftedSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, val, b, sigma, ptr, col, seed, params):
        # the library works on its own stream: torch's pending work first
        torch.cuda.current_stream().synchronize()
        cx = Context()
        A = Matrix(cx, ptr, col, val)
        m, n = int(sigma.shape[0]), int(b.shape[0])
        X = torch.empty((m, n), dtype=torch.float64, device=b.device)
        res = Solver(A, m, **params).run(b, sigma, seed=seed, x=X)
        torch.cuda.current_stream().synchronize()
        ctx.save_for_backward(val, sigma, X)
        ctx.ptr, ctx.col, ctx.seed, ctx.params, ctx.k = ptr, col, seed, params, res.k
        return X

    @staticmethod
    def backward(ctx, G):
        val, sigma, X = ctx.saved_tensors
        G = G.contiguous()
        torch.cuda.current_stream().synchronize()
        cx = Context()
        A = Matrix(cx, ctx.ptr, ctx.col, val)
        At = A.transpose()
        m, n = X.shape
        r1 = _rank_one(G)
        if r1 is not None:
            w, g = r1
            w, g = w.contiguous(), g.contiguous()
            Y = torch.empty((m, n), dtype=torch.float64, device=G.device)
            torch.cuda.current_stream().synchronize()
            Solver(At, m, **ctx.params).run(g, sigma, seed=ctx.seed, x=Y)
            dval, db, ds = A.adjoint_gradients(X, Y, w)
        else:
            Lam = torch.zeros((m, n), dtype=torch.float64, device=G.device)
            torch.cuda.current_stream().synchronize()
            for j in range(m):
                if float(torch.max(torch.abs(G[j]))) == 0.0:
                    continue
                Solver(At, 1, **ctx.params).run(G[j].contiguous(), sigma[j:j + 1].contiguous(), seed=0,
                                                x=Lam[j:j + 1])
            dval, db, ds = A.adjoint_gradients(X, Lam)
        torch.cuda.current_stream().synchronize()
        return dval, db, ds, None, None, None, None


def shifted_solve(ptr, col, val, b, sigma, seed: int = 0, **params):
    params.setdefault("tol", 1e-12)
    params.setdefault("max_iter", 10000)
    return _ShiftedSolve.apply(val, b, sigma, ptr, col, int(seed), params)
