"""Synthetic workload generators: sizes and properties of the named shapes."""
import numpy as np


def test_stencil_sizes(pkg):
    a = pkg.workloads.stencil_cd3d(32)
    assert a.n == 32768 and a.nnz == 223232  # 7 N^3 - 6 N^2
    assert a.ptr.dtype == np.uint32 and a.col.dtype == np.uint32 and a.val.dtype == np.float64
    d = pkg.workloads.stencil_cd2d(10)
    assert d.n == 100 and d.nnz == 5 * 100 - 4 * 10


def test_stencil_values_and_order(pkg):
    a = pkg.workloads.stencil_cd3d(4)
    i = 1 + 4 * (1 + 4 * 1)  # interior point (1,1,1)
    cols = a.col[a.ptr[i]:a.ptr[i + 1]].astype(int)
    vals = a.val[a.ptr[i]:a.ptr[i + 1]]
    assert list(cols) == [i - 16, i - 4, i - 1, i, i + 1, i + 4, i + 16]
    assert list(vals) == [-1.0, -1.0, -1.2, 6.0, -0.8, -1.0, -1.0]
    assert np.all(np.diff(a.col[a.ptr[0]:a.ptr[1]].astype(int)) > 0)


def test_irregular_powerlaw(pkg):
    a = pkg.workloads.irregular_powerlaw(20000, seed=0)
    lens = np.diff(a.ptr.astype(np.int64))
    assert 13.0 < lens.mean() < 17.0 and lens.max() <= 4000 and lens.min() >= 1
    rows = np.repeat(np.arange(a.n), lens)
    diag = a.val[a.col == rows]
    off = np.bincount(rows, weights=np.abs(a.val) * (a.col != rows), minlength=a.n)
    assert diag.shape[0] == a.n and np.all(diag > off)  # strictly diagonally dominant
    b = pkg.workloads.irregular_powerlaw(20000, seed=0)
    assert np.array_equal(a.col, b.col) and np.array_equal(a.val, b.val)


def test_named_families(pkg):
    f = pkg.workloads.family("c1")
    assert f.a.n == 32768 and len(f.sigma) == 16 and f.sigma[15] == 0.15 and f.tol == 1e-10
    f = pkg.workloads.family("c2", scale=16)
    assert len(f.sigma) == 64 and abs(f.sigma[0] - 1e-4) < 1e-18 and abs(f.sigma[-1] - 1.0) < 1e-12
    assert abs(np.linalg.norm(f.b) - 1.0) < 1e-12


def test_batched_families(pkg):
    fams = pkg.workloads.batched_families(12, seed=0)
    assert len(fams) == 12
    for f in fams:
        assert 8 <= len(f.sigma) <= 64 and np.all(np.diff(f.sigma) >= 0)
        assert 0.5e4 <= f.a.n <= 1e6


def test_transpose(pkg):
    a = pkg.workloads.irregular_powerlaw(300, mean_len=6, max_len=40, seed=1)
    t = a.transpose()
    assert np.allclose(t.to_dense(), a.to_dense().T, rtol=0, atol=0)
