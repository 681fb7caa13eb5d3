"""CSR SpMV kernel parity: bit-exact against the oracle's stored-order FMA row
sums for every row a single thread sums (SELL-32 and HYB slice rows, rows
staged in shared memory in the tile form); rows summed by a warp or a block
(a fixed tree over lanes) and the reference's non-FMA row sums within
rounding."""
import numpy as np
import pytest

from conftest import GoldenCsr, golden

pytestmark = pytest.mark.gpu


def _gpu_spmv(pkg, a, x, sigma=0.0, fmt=None, want_fmt=None):
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    if fmt:
        A.set_format(fmt)
    if want_fmt:
        assert A.format == want_fmt
    y = np.zeros(a.n)
    A.spmv(np.ascontiguousarray(x, dtype=np.float64), y, sigma)
    A.close()
    ctx.close()
    return y


def test_stencil_bitwise(cuda, pkg, oracle):
    a = pkg.workloads.stencil_cd3d(40, 33, 17)
    x = np.random.default_rng(0).standard_normal(a.n)
    assert np.array_equal(_gpu_spmv(pkg, a, x), oracle.spmv_fma(a, x))


@pytest.mark.parametrize("fmt,single", [(None, 32), ("tile", 256)], ids=["hyb-default", "tile"])
def test_irregular_short_rows_bitwise_long_rows_close(cuda, pkg, oracle, fmt, single):
    """Power-law rows: by default the HYB form (rows of <= 32 entries in
    length-sorted SELL-32 slices, longer rows one warp each); the tile form on
    request (rows of <= 256 entries in shared-memory tiles)."""
    a = pkg.workloads.irregular_powerlaw(200000, seed=2)
    x = np.random.default_rng(1).standard_normal(a.n)
    y = _gpu_spmv(pkg, a, x, fmt=fmt, want_fmt=fmt or "hyb")
    want = oracle.spmv_fma(a, x)
    lens = np.diff(a.ptr.astype(np.int64))
    short = lens <= single  # rows one thread sums in stored order: same bits
    assert short.sum() > 0 and (~short).sum() > 0
    assert np.array_equal(y[short], want[short])
    scale = np.abs(a.val).max() * np.abs(x).max() * lens[~short]
    assert np.all(np.abs(y[~short] - want[~short]) <= 1e-15 * scale)


def _random_csr(pkg, n, lens, seed):
    rng = np.random.default_rng(seed)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    np.cumsum(lens, out=ptr[1:])
    col = rng.integers(0, n, int(ptr[-1])).astype(np.uint32)
    val = rng.standard_normal(int(ptr[-1]))
    return pkg.workloads.Csr(ptr, col, val)


@pytest.mark.parametrize("case", ["window_edges", "all_long", "all_short_padded", "empty_windows"])
def test_hyb_shapes(cuda, pkg, oracle, case):
    """HYB edge cases: n not a multiple of the 256-row window, only warp rows,
    only slice rows (SELL-32 rejected for its padding), whole windows of empty
    rows."""
    rng = np.random.default_rng(len(case))
    if case == "window_edges":
        n = 256 * 7 + 37
        lens = rng.choice([0, 1, 3, 31, 32, 33, 70, 600], size=n)
    elif case == "all_long":
        n = 300
        lens = rng.integers(33, 900, n)
    elif case == "all_short_padded":
        n = 5000
        lens = np.where(rng.random(n) < 0.05, 30, 1)
    else:
        n = 256 * 4
        lens = np.zeros(n, dtype=np.int64)
        lens[256:512] = rng.integers(0, 40, 256)
    a = _random_csr(pkg, n, lens, seed=3)
    x = rng.standard_normal(n)
    y = _gpu_spmv(pkg, a, x, fmt="hyb", want_fmt="hyb")
    want = oracle.spmv_fma(a, x)
    short = lens <= 32
    assert np.array_equal(y[short], want[short])
    scale = np.abs(a.val).max(initial=0.0) * np.abs(x).max() * np.maximum(lens, 1)
    assert np.all(np.abs(y - want) <= 1e-15 * scale)


def test_format_switching_same_products(cuda, pkg, oracle):
    a = pkg.workloads.irregular_powerlaw(30000, seed=4)
    x = np.random.default_rng(2).standard_normal(a.n)
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    assert A.format == "hyb"
    ys = {}
    for fmt in ["tile", "hyb", "tile", "hyb"]:
        A.set_format(fmt)
        assert A.format == fmt
        y = np.zeros(a.n)
        A.spmv(x, y, 0.25)
        ys.setdefault(fmt, []).append(y)
    A.close()
    ctx.close()
    assert np.array_equal(ys["tile"][0], ys["tile"][1]) and np.array_equal(ys["hyb"][0], ys["hyb"][1])
    want = oracle.spmv_fma(a, x) + 0.25 * x
    for y in (ys["tile"][0], ys["hyb"][0]):
        assert np.max(np.abs(y - want)) <= 1e-13 * np.max(np.abs(want))


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
