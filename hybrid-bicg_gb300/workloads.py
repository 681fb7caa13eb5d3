"""Synthetic shifted families of the shapes the solver is measured on.

The reference ships no matrices (its job scripts name SuiteSparse files that are
not part of it, e.g. run_grand.bash:12), so every workload here is generated,
seeded and deterministic.  All matrices are square CSR with 32-bit unsigned
row pointers and column indices (the reference's CSR_Matrix, src/matrix.h:19-26)
and FP64 values; inside a row the columns are ascending, which is also the order
a Matrix Market file written from them keeps (src/matrix.c:176-232 sorts rows
stably and leaves each row in file order).

Workloads:
  c1  32^3 convection-diffusion, 16 shifts sigma_k = 0.01 k, b = 1/sqrt(n)
  c2  256^3 convection-diffusion, 64 shifts geometric in [1e-4, 1], b ~ N(0,1) normalised
  c3  n = 2M power-law rows (Zipf 2.0, mean 16, clipped [1, 4000]), 32 shifts in [0, 0.5]
  c4  256 families of 2-D 5-point / 3-D 7-point stencils, n log-uniform in [1e4, 5e5]
  c5  128^3 convection-diffusion, 32 shifts in [1e-3, 1], adjoint weights w, c
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Csr", "Family", "stencil_cd3d", "stencil_cd2d", "irregular_powerlaw", "family", "batched_families",
    "adjoint_problem", "write_matrix_market",
]


@dataclass
class Csr:
    """Square CSR matrix: ptr (n+1, uint32), col (nnz, uint32), val (nnz, float64)."""

    ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray

    @property
    def n(self) -> int:
        return int(self.ptr.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.ptr[-1])

    def to_dense(self) -> np.ndarray:
        n = self.n
        a = np.zeros((n, n))
        rows = np.repeat(np.arange(n), np.diff(self.ptr.astype(np.int64)))
        np.add.at(a, (rows, self.col.astype(np.int64)), self.val)
        return a

    def matvec(self, x: np.ndarray) -> np.ndarray:
        rows = np.repeat(np.arange(self.n), np.diff(self.ptr.astype(np.int64)))
        return np.bincount(rows, weights=self.val * x[self.col], minlength=self.n)

    def transpose(self) -> "Csr":
        n = self.n
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(self.ptr.astype(np.int64)))
        cols = self.col.astype(np.int64)
        order = np.lexsort((rows, cols))
        counts = np.bincount(cols, minlength=n)
        ptr = np.zeros(n + 1, dtype=np.uint32)
        np.cumsum(counts, out=ptr[1:])
        return Csr(ptr, rows[order].astype(np.uint32), self.val[order].copy())


@dataclass
class Family:
    """One shifted family (A + sigma_j I) x_j = b plus its solve settings."""

    name: str
    a: Csr
    b: np.ndarray
    sigma: np.ndarray
    seed: int = 0
    tol: float = 1e-10
    max_iter: int = 10000
    extra: dict = field(default_factory=dict)


def _stencil(dims: tuple[int, ...], diag: float, west: float, east: float, other: float) -> Csr:
    """Natural-order (first index fastest) convection-diffusion stencil.

    Rows list their neighbours in ascending column order: the slowest axis
    first, the x neighbours around the diagonal.  Neighbours outside the grid
    are dropped (homogeneous Dirichlet boundary)."""
    n = int(np.prod(dims))
    idx = np.arange(n, dtype=np.int64)
    coords = []
    rem = idx
    for d in dims:
        coords.append(rem % d)
        rem = rem // d
    offsets, values, masks = [], [], []
    stride = [1]
    for d in dims[:-1]:
        stride.append(stride[-1] * d)
    # slow axes (descending) below the diagonal, then x west / diag / x east, then slow axes above
    for ax in reversed(range(1, len(dims))):
        offsets.append(-stride[ax]); values.append(other); masks.append(coords[ax] > 0)
    offsets.append(-1); values.append(west); masks.append(coords[0] > 0)
    offsets.append(0); values.append(diag); masks.append(np.ones(n, dtype=bool))
    offsets.append(1); values.append(east); masks.append(coords[0] < dims[0] - 1)
    for ax in range(1, len(dims)):
        offsets.append(stride[ax]); values.append(other); masks.append(coords[ax] < dims[ax] - 1)
    mask = np.stack(masks, axis=1)
    counts = mask.sum(axis=1)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    np.cumsum(counts, out=ptr[1:])
    col = (idx[:, None] + np.asarray(offsets, dtype=np.int64)[None, :])[mask].astype(np.uint32)
    val = np.broadcast_to(np.asarray(values, dtype=np.float64)[None, :], mask.shape)[mask].copy()
    return Csr(ptr, col, val)


def stencil_cd3d(nx: int, ny: int | None = None, nz: int | None = None, diag: float = 6.0, west: float = -1.2,
                 east: float = -0.8, other: float = -1.0) -> Csr:
    """3-D 7-point convection-diffusion: diagonal 6, x neighbours -1 -+ 0.2 (upwind,
    Peclet 0.2), y/z neighbours -1.  32^3 gives n = 32768, nnz = 223232."""
    return _stencil((nx, ny or nx, nz or nx), diag, west, east, other)


def stencil_cd2d(nx: int, ny: int | None = None, diag: float = 4.0, west: float = -1.2, east: float = -0.8,
                 other: float = -1.0) -> Csr:
    """2-D 5-point convection-diffusion with the same x convection as the 3-D one."""
    return _stencil((nx, ny or nx), diag, west, east, other)


def irregular_powerlaw(n: int, mean_len: float = 16.0, max_len: int = 4000, zipf_a: float = 2.0,
                       band: int = 64, band_frac: float = 0.3, seed: int = 0) -> Csr:
    """Random nonsymmetric matrix with power-law row lengths.

    Row lengths (diagonal included) are Zipf(zipf_a) draws scaled so that the
    mean after clipping to [1, max_len] is mean_len.  Off-diagonal columns are
    uniform on [0, n) with probability 1 - band_frac, else uniform within
    +-band of the row; duplicates and the diagonal are removed.  Off-diagonal
    values are N(0,1); the diagonal is 1.1 x the row's absolute off-diagonal
    sum (1.0 for a row with no off-diagonal entry), so A is strictly
    diagonally dominant.  Removing duplicate columns shortens rows (most of all
    the long ones, whose near-diagonal draws collide in the +-band window), so
    the drawn lengths aim at a mean that is raised until the mean after
    de-duplication is mean_len (within 0.5 %, at most six passes)."""
    aim = mean_len
    for _ in range(6):
        a = _powerlaw_draw(n, aim, mean_len, max_len, zipf_a, band, band_frac, seed)
        got = a.nnz / n
        if abs(got - mean_len) <= 0.005 * mean_len:
            break
        aim *= mean_len / got
    return a


def _powerlaw_draw(n: int, aim: float, mean_len: float, max_len: int, zipf_a: float, band: int, band_frac: float,
                   seed: int) -> Csr:
    """One draw of irregular_powerlaw with the row lengths (before duplicate
    columns are removed) scaled to mean `aim`."""
    rng = np.random.default_rng(seed)
    z = rng.zipf(zipf_a, size=n).astype(np.float64)
    z = np.minimum(z, float(max_len))
    lo, hi = 0.01, 1000.0
    for _ in range(60):
        c = 0.5 * (lo + hi)
        mean = np.clip(np.rint(c * z), 1, max_len).mean()
        if mean < aim:
            lo = c
        else:
            hi = c
    lens = np.clip(np.rint(0.5 * (lo + hi) * z), 1, max_len).astype(np.int64)
    n_off = lens - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), n_off)
    tot = rows.shape[0]
    in_band = rng.random(tot) < band_frac
    cols = rng.integers(0, n, size=tot, dtype=np.int64)
    cols_band = rows + rng.integers(-band, band + 1, size=tot, dtype=np.int64)
    cols = np.where(in_band, np.clip(cols_band, 0, n - 1), cols)
    keep = cols != rows
    key = np.sort(rows[keep] * n + cols[keep])
    key = key[np.concatenate(([True], key[1:] != key[:-1]))] if key.size else key
    rows_o, cols_o = key // n, key % n
    vals_o = rng.standard_normal(rows_o.shape[0])
    absrow = np.bincount(rows_o, weights=np.abs(vals_o), minlength=n)
    diag = np.where(absrow > 0, 1.1 * absrow, 1.0)
    all_rows = np.concatenate([rows_o, np.arange(n, dtype=np.int64)])
    all_cols = np.concatenate([cols_o, np.arange(n, dtype=np.int64)])
    all_vals = np.concatenate([vals_o, diag])
    order = np.argsort(all_rows * n + all_cols, kind="stable")
    counts = np.bincount(all_rows, minlength=n)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    np.cumsum(counts, out=ptr[1:])
    return Csr(ptr, all_cols[order].astype(np.uint32), all_vals[order])


def _normal_rhs(n: int, seed: int) -> np.ndarray:
    b = np.random.default_rng(seed).standard_normal(n)
    return b / np.linalg.norm(b)


def family(name: str, scale: int | None = None) -> Family:
    """The named single-family workload.  `scale` overrides the grid side
    (c1/c2/c5) or n (c3) to make small cases of the same shape for tests."""
    if name == "c1":
        side = scale or 32
        a = stencil_cd3d(side)
        b = np.full(a.n, 1.0 / np.sqrt(a.n))
        return Family("c1", a, b, 0.01 * np.arange(16, dtype=np.float64), seed=0, tol=1e-10, max_iter=10000)
    if name == "c2":
        side = scale or 256
        a = stencil_cd3d(side)
        sigma = 1e-4 * 10.0 ** (4.0 * np.arange(64) / 63.0)
        return Family("c2", a, _normal_rhs(a.n, 0), sigma, seed=0, tol=1e-10, max_iter=10000)
    if name == "c3":
        n = scale or 2_000_000
        a = irregular_powerlaw(n, seed=0)
        sigma = np.sort(np.random.default_rng(0).uniform(0.0, 0.5, 32))
        return Family("c3", a, _normal_rhs(a.n, 1), sigma, seed=0, tol=1e-10, max_iter=10000)
    if name == "c5":
        side = scale or 128
        return adjoint_problem(side)
    raise ValueError(f"unknown workload {name!r}")


def batched_families(count: int = 256, n_lo: float = 1e4, n_hi: float = 5e5, seed: int = 0) -> list[Family]:
    """Uneven families: even index -> 2-D 5-point, odd -> 3-D 7-point; grid side
    chosen so n is log-uniform in [n_lo, n_hi]; 8..64 shifts uniform in
    [1e-3, 1] (sorted, seed = the smallest); b ~ N(0,1) with seed f."""
    rng = np.random.default_rng(seed)
    fams = []
    for f in range(count):
        target = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        if f % 2 == 0:
            side = max(2, int(round(np.sqrt(target))))
            a = stencil_cd2d(side)
        else:
            side = max(2, int(round(target ** (1.0 / 3.0))))
            a = stencil_cd3d(side)
        m = int(rng.integers(8, 65))
        sigma = np.sort(rng.uniform(1e-3, 1.0, m))
        b = np.random.default_rng(1000 + f).standard_normal(a.n)
        fams.append(Family(f"c4/{f}", a, b, sigma, seed=0, tol=1e-10, max_iter=10000))
    return fams


def adjoint_problem(side: int = 128, m: int = 32, seed: int = 0) -> Family:
    """J = sum_k w_k c^T x(sigma_k) on a side^3 convection-diffusion matrix:
    32 shifts uniform in [1e-3, 1], w ~ U(0,1), b and c ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    a = stencil_cd3d(side)
    sigma = np.sort(rng.uniform(1e-3, 1.0, m))
    w = rng.uniform(0.0, 1.0, m)
    b = rng.standard_normal(a.n)
    c = rng.standard_normal(a.n)
    return Family("c5", a, b, sigma, seed=0, tol=1e-10, max_iter=10000, extra={"w": w, "c": c})


def write_matrix_market(path: str, a: Csr, comment: str = "") -> None:
    """Write `a` as 'matrix coordinate real general', one 1-based triplet per
    line in CSR order (row-major, columns as stored)."""
    n = a.n
    rows = np.repeat(np.arange(1, n + 1, dtype=np.int64), np.diff(a.ptr.astype(np.int64)))
    with open(path, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate real general\n")
        if comment:
            for line in comment.splitlines():
                fh.write(f"% {line}\n")
        fh.write(f"{n} {n} {a.nnz}\n")
        data = np.empty(a.nnz, dtype=[("r", np.int64), ("c", np.int64), ("v", np.float64)])
        data["r"] = rows
        data["c"] = a.col.astype(np.int64) + 1
        data["v"] = a.val
        np.savetxt(fh, data, fmt="%d %d %.17g")
