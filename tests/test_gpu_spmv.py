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


def _hyb_window():
    """The HYB sort window (HBK_HYB_WINDOW in the kernels' header)."""
    import re
    from pathlib import Path

    text = (Path(__file__).resolve().parents[1] / "hybrid-bicg_gb300" / "csrc" / "hbk.h").read_text()
    return int(re.search(r"#define HBK_HYB_WINDOW (\d+)", text).group(1))


@pytest.mark.parametrize("case", ["window_edges", "all_long", "all_short_padded", "empty_windows",
                                  "few_huge_rows", "more_items_than_warps", "lane_class_edges"])
def test_hyb_shapes(cuda, pkg, oracle, case):
    """HYB edge cases: n not a multiple of the sort window, only long rows,
    only slice rows (SELL-32 rejected for its padding), whole windows of empty
    rows, a few rows far longer than the rest (each alone in a warp's list),
    many more work items than warps (long lists), and long rows at the edges
    of the 4-, 16- and 32-lane classes with counts that leave a partial group
    of 8 rows and a partial pair."""
    rng = np.random.default_rng(len(case))
    win = _hyb_window()
    if case == "window_edges":
        n = win * 7 + 37
        lens = rng.choice([0, 1, 3, 31, 32, 33, 70, 600], size=n)
    elif case == "all_long":
        n = 300
        lens = rng.integers(33, 900, n)
    elif case == "all_short_padded":
        n = 5000
        lens = np.where(rng.random(n) < 0.05, 30, 1)
    elif case == "few_huge_rows":
        n = 40000
        lens = rng.integers(0, 12, n)
        lens[rng.choice(n, 5, replace=False)] = 20000
    elif case == "lane_class_edges":
        n = 3001
        lens = rng.choice([0, 5, 32], size=n)
        edges = [33] * 13 + [128] * 5 + [129] * 3 + [512] * 7 + [513] * 1 + [2000] * 2
        lens[rng.choice(n, len(edges), replace=False)] = edges
    elif case == "more_items_than_warps":
        n = 600000
        lens = np.where(rng.random(n) < 0.03, rng.integers(33, 300, n), rng.integers(0, 9, n))
    else:
        n = win * 4
        lens = np.zeros(n, dtype=np.int64)
        lens[win:2 * win] = rng.integers(0, 40, win)
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


# ---- MERGE form: nonzero-balanced blocks (merge-path split among threads)
MERGE_IPT, MERGE_ITEMS = 8, 32 * 8
MERGE_LONG = MERGE_ITEMS - 1


def merge_whole_rows(ptr):
    """Rows the MERGE form sums in one lane (same bits as the stored-order
    FMA sum): the host plan (blocks of consecutive rows of <= 255 entries with
    rows + nonzeros <= 256, one warp each, cut before every longer row)
    restated, then inside a block row i's nonzeros are merge items i +
    ptr-offsets and its end item i + end offset; the row is whole when its
    first nonzero and its end item fall in the same lane's run of 8 items.
    Empty rows are exact zeros whoever ends them."""
    lens = np.diff(ptr.astype(np.int64))
    n = lens.shape[0]
    whole = np.zeros(n, dtype=bool)
    blocks, open_, items, r0 = [], False, 0, 0
    for r in range(n):
        ln = int(lens[r])
        if ln > MERGE_LONG:
            if open_:
                blocks.append((r0, r))
            open_ = False
            continue
        if not open_ or items + ln + 1 > MERGE_ITEMS:
            if open_:
                blocks.append((r0, r))
            r0, open_, items = r, True, 0
        items += ln + 1
    if open_:
        blocks.append((r0, n))
    for (a, b) in blocks:
        rel_end = ptr[a + 1:b + 1].astype(np.int64) - int(ptr[a])
        rel_start = ptr[a:b].astype(np.int64) - int(ptr[a])
        i = np.arange(b - a)
        first = (i + rel_start) // MERGE_IPT
        last = (i + rel_end) // MERGE_IPT
        whole[a:b] = (first == last) | (rel_end == rel_start)
    return whole, lens > MERGE_LONG


def _check_merge(y, want, a, x):
    whole, long_ = merge_whole_rows(a.ptr)
    assert np.array_equal(y[whole], want[whole])
    lens = np.diff(a.ptr.astype(np.int64))
    scale = np.abs(a.val).max(initial=0.0) * np.abs(x).max() * np.maximum(lens, 1)
    assert np.all(np.abs(y - want) <= 1e-15 * scale)
    return whole, long_


def test_merge_powerlaw(cuda, pkg, oracle):
    """Power-law rows in the MERGE form: rows a thread sums whole are
    bit-exact, rows cut between threads (a sum of stored-order FMA pieces in
    thread order) and long rows (one warp, fixed tree) within rounding."""
    a = pkg.workloads.irregular_powerlaw(200000, seed=2)
    x = np.random.default_rng(1).standard_normal(a.n)
    y = _gpu_spmv(pkg, a, x, fmt="merge", want_fmt="merge")
    whole, long_ = _check_merge(y, oracle.spmv_fma(a, x), a, x)
    assert whole.sum() > 0.2 * a.n and (~whole & ~long_).sum() > 0 and long_.sum() > 0


@pytest.mark.parametrize("case", ["boundaries", "all_long", "all_empty", "one_row", "full_blocks", "mixed_empty"])
def test_merge_shapes(cuda, pkg, oracle, case):
    """MERGE edge cases: rows of exactly 255 and 256 entries (the long-row
    limit: a row and its end fill a warp's block), rows cut across many lanes,
    blocks filled to the last item, only long rows (one warp each, lengths
    around the four-chain stride), only empty rows, a single row, runs of empty
    rows between long ones."""
    rng = np.random.default_rng(len(case) + 11)
    if case == "boundaries":
        n = 3000
        lens = rng.choice([0, 1, 5, 7, 8, 9, 31, 32, 33, 100, 254, 255, 256, 257, 4000], size=n)
    elif case == "all_long":
        n = 200
        lens = rng.choice([256, 300, 383, 384, 385, 511, 512, 513, 2000, 6000], size=n)
    elif case == "all_empty":
        n = 4000
        lens = np.zeros(n, dtype=np.int64)
    elif case == "one_row":
        n = 1
        lens = np.array([1])
    elif case == "full_blocks":
        n = 64
        lens = np.full(n, 31)  # 8 rows x 32 items = one full block
    else:
        n = 5000
        lens = np.where(rng.random(n) < 0.02, 2000, 0)
        lens[rng.random(n) < 0.3] = 3
        lens[rng.random(n) < 0.05] = 150
    a = _random_csr(pkg, n, lens, seed=5)
    x = rng.standard_normal(n)
    y = _gpu_spmv(pkg, a, x, fmt="merge", want_fmt="merge")
    _check_merge(y, oracle.spmv_fma(a, x), a, x)


def test_merge_in_the_solver(cuda, pkg, oracle):
    """A shifted solve with the matrix in the MERGE form (fused, incremental
    and deferred) reaches the reference's solutions."""
    g = golden("irregular_fixed_seed")
    a = GoldenCsr(g)
    for mode in ("incremental", "deferred"):
        ctx = pkg.Context()
        A = pkg.Matrix(ctx, a.ptr, a.col, a.val)
        A.set_format("merge")
        s = pkg.Solver(A, len(g["sigma"]), tol=float(g["tol"]), max_iter=int(g["max_iter"]),
                       switching=bool(g["switching"]), shift_mode=mode, refine=False)
        res = s.run(g["b"], g["sigma"], seed=int(g["seed"]))
        s.close()
        A.close()
        ctx.close()
        err = np.max(np.abs(np.asarray(res.x) - g["x"])) / np.max(np.abs(g["x"]))
        assert err < 1e-8, (mode, err)
