"""GPU COO -> CSR (hbicg_matrix_from_coo, hbicg_matrix_load_mm): the row
order of the reference's coo2csr (stable: entries of a row keep their given
order), bit for bit, against the reference's loader outputs and a numpy
stable sort; radix passes for 1, 2, 3 and 4 bytes of row index."""
import numpy as np
import pytest
from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu

MM_NAMES = ["mm_real_general.mtx", "mm_integer.mtx", "mm_pattern.mtx", "mm_symmetric.mtx", "mm_upper_banner.mtx"]


def _stable_csr(n, row, col, val):
    order = np.argsort(row, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, row.astype(np.int64) + 1, 1)
    return np.cumsum(ptr).astype(np.uint32), col[order], val[order]


@pytest.mark.parametrize("name", MM_NAMES)
def test_load_mm_matches_reference_loader(cuda, pkg, name):
    g = golden("mm_loader")
    ctx = pkg.Context()
    A = pkg.Matrix.load_mm(ctx, str(GOLDEN / name))
    ptr, col, val = A.csr()
    assert np.array_equal(ptr, g[f"{name}:ptr"]) and np.array_equal(col, g[f"{name}:col"])
    assert np.array_equal(val, g[f"{name}:val"])
    A.close()


def _coo(n, nnz, seed, long_row=None):
    rng = np.random.default_rng(seed)
    row = rng.integers(0, n, nnz).astype(np.uint32)
    if long_row is not None:
        row[rng.random(nnz) < 0.3] = long_row  # one very long row
    col = rng.integers(0, n, nnz).astype(np.uint32)
    val = rng.standard_normal(nnz)
    return row, col, val


@pytest.mark.parametrize("n,nnz,long_row", [
    (1, 5, None),            # one row, one pass
    (200, 3000, None),       # one pass, many tiles share digits
    (50000, 400000, 17),     # two passes, empty rows, a 120k-entry row
    (3000000, 500000, None),  # three passes, mostly empty rows
    (20000000, 300000, 19999999),  # four passes (rows above 2^24), a long last row
])
def test_from_coo_matches_stable_sort(cuda, pkg, n, nnz, long_row):
    row, col, val = _coo(n, nnz, seed=n % 97, long_row=long_row)
    ctx = pkg.Context()
    A = pkg.Matrix.from_coo(ctx, n, row, col, val)
    ptr, c, v = A.csr()
    eptr, ecol, evl = _stable_csr(n, row, col, val)
    assert np.array_equal(ptr, eptr)
    assert np.array_equal(c, ecol) and np.array_equal(v, evl)
    A.close()


def test_from_coo_four_byte_rows(cuda, pkg):
    """Row indices above 2^24 (a fourth radix pass); few entries, device input."""
    torch = cuda
    n = (1 << 25) + 3
    rng = np.random.default_rng(5)
    row = np.concatenate([rng.integers(0, n, 20000), np.full(50, n - 1), np.zeros(50)]).astype(np.uint32)
    col = rng.integers(0, n, row.size).astype(np.uint32)
    val = rng.standard_normal(row.size)
    ctx = pkg.Context()
    A = pkg.Matrix.from_coo(ctx, n, torch.from_numpy(row.astype(np.int32)).cuda(),
                            torch.from_numpy(col.astype(np.int32)).cuda(), torch.from_numpy(val).cuda())
    ptr, c, v = A.csr()
    eptr, ecol, evl = _stable_csr(n, row, col, val)
    assert np.array_equal(ptr, eptr) and np.array_equal(c, ecol) and np.array_equal(v, evl)
    A.close()


def test_from_coo_empty_and_bad_index(cuda, pkg):
    ctx = pkg.Context()
    z = np.zeros(0, dtype=np.uint32)
    A = pkg.Matrix.from_coo(ctx, 10, z, z, np.zeros(0))
    ptr, c, v = A.csr()
    assert np.array_equal(ptr, np.zeros(11, np.uint32)) and c.size == 0
    A.close()
    with pytest.raises(RuntimeError, match="index"):
        pkg.Matrix.from_coo(ctx, 10, np.array([1, 10], np.uint32), np.array([0, 0], np.uint32), np.ones(2))


def test_solve_on_loaded_matrix_matches(cuda, pkg, tmp_path):
    """A family solved on a matrix read from its Matrix Market file and built
    on the GPU equals the solve on the same CSR given directly."""
    a = pkg.workloads.stencil_cd3d(10)
    path = tmp_path / "a.mtx"
    pkg.workloads.write_matrix_market(str(path), a)
    b = np.full(a.n, 1.0 / np.sqrt(a.n))
    sigma = 0.01 * np.arange(8, dtype=np.float64)
    ctx = pkg.Context()
    A1 = pkg.Matrix(ctx, a.ptr, a.col, a.val)
    A2 = pkg.Matrix.load_mm(ctx, str(path))
    assert np.array_equal(A2.csr()[0], a.ptr.astype(np.uint32)) and np.array_equal(A2.csr()[2], a.val)
    r1 = pkg.Solver(A1, len(sigma), tol=1e-10, max_iter=1000).run(b, sigma, seed=0)
    r2 = pkg.Solver(A2, len(sigma), tol=1e-10, max_iter=1000).run(b, sigma, seed=0)
    assert r1.k == r2.k and np.array_equal(r1.x, r2.x)
