"""CSR SpMV kernel parity: bit-exact against the oracle's stored-order FMA row
sums for rows staged in shared memory; long rows (block tree reduction) and the
reference's non-FMA row sums within rounding."""
import numpy as np
import pytest

from conftest import GoldenCsr, golden

pytestmark = pytest.mark.gpu


def _gpu_spmv(pkg, a, x, sigma=0.0):
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    y = np.zeros(a.n)
    A.spmv(np.ascontiguousarray(x, dtype=np.float64), y, sigma)
    A.close()
    ctx.close()
    return y


def test_stencil_bitwise(cuda, pkg, oracle):
    a = pkg.workloads.stencil_cd3d(40, 33, 17)
    x = np.random.default_rng(0).standard_normal(a.n)
    assert np.array_equal(_gpu_spmv(pkg, a, x), oracle.spmv_fma(a, x))


def test_irregular_short_rows_bitwise_long_rows_close(cuda, pkg, oracle):
    a = pkg.workloads.irregular_powerlaw(200000, seed=2)
    x = np.random.default_rng(1).standard_normal(a.n)
    y = _gpu_spmv(pkg, a, x)
    want = oracle.spmv_fma(a, x)
    lens = np.diff(a.ptr.astype(np.int64))
    short = lens <= 256  # rows of a shared-memory tile: same order, same bits
    assert short.sum() > 0 and (~short).sum() > 0
    assert np.array_equal(y[short], want[short])
    scale = np.abs(a.val).max() * np.abs(x).max() * lens[~short]
    assert np.all(np.abs(y[~short] - want[~short]) <= 1e-15 * scale)


def test_against_reference_golden(cuda, pkg):
    g = golden("spmv_irregular")
    y = _gpu_spmv(pkg, GoldenCsr(g), g["x"])
    assert np.max(np.abs(y - g["y"])) <= 1e-13 * np.max(np.abs(g["y"]))


def test_shifted_product(cuda, pkg, oracle):
    a = pkg.workloads.stencil_cd2d(64)
    x = np.random.default_rng(4).standard_normal(a.n)
    y = _gpu_spmv(pkg, a, x, sigma=0.37)
    want = oracle.spmv_fma(a, x) + 0.37 * x
    assert np.max(np.abs(y - want)) <= 1e-14 * np.max(np.abs(want))


def test_empty_rows_and_tiny(cuda, pkg, oracle):
    n = 1000
    rng = np.random.default_rng(5)
    lens = rng.integers(0, 4, n)
    lens[::7] = 0
    ptr = np.zeros(n + 1, dtype=np.uint32)
    np.cumsum(lens, out=ptr[1:])
    col = rng.integers(0, n, int(ptr[-1])).astype(np.uint32)
    val = rng.standard_normal(int(ptr[-1]))
    a = pkg.workloads.Csr(ptr, col, val)
    x = rng.standard_normal(n)
    assert np.array_equal(_gpu_spmv(pkg, a, x), oracle.spmv_fma(a, x))
    one = pkg.workloads.Csr(np.array([0, 1], np.uint32), np.array([0], np.uint32), np.array([2.5]))
    assert _gpu_spmv(pkg, one, np.array([4.0]))[0] == 10.0


def test_single_very_long_row(cuda, pkg):
    n = 5000
    ptr = np.zeros(n + 1, dtype=np.uint32)
    ptr[1:] = n  # row 0 holds every column, the other rows are empty
    col = np.arange(n, dtype=np.uint32)
    val = np.random.default_rng(6).standard_normal(n)
    a = pkg.workloads.Csr(ptr, col, val)
    x = np.random.default_rng(7).standard_normal(n)
    y = _gpu_spmv(pkg, a, x)
    assert abs(y[0] - np.dot(val, x)) <= 1e-12 * np.abs(val * x).sum()
    assert np.all(y[1:] == 0.0)


def test_dropin_mult_accumulates(cuda, pkg, oracle):
    a = pkg.workloads.stencil_cd3d(9)
    x = np.random.default_rng(8).standard_normal(a.n)
    y0 = np.random.default_rng(9).standard_normal(a.n)
    y = pkg.mult(a, x, y0.copy())
    assert np.max(np.abs(y - (y0 + oracle.spmv_fma(a, x)))) <= 1e-14 * np.max(np.abs(y))
