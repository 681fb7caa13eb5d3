"""Parallel Matrix Market reader (hbicg_mm_read) against the reference's own
loader outputs (tests/golden/mm_loader.npz, made by running the reference's
src/matrix.c through tests/golden/make_golden.py) and against a plain Python
parse of the same text; no GPU needed."""
import numpy as np
import pytest
from conftest import GOLDEN, golden

MM_NAMES = ["mm_real_general.mtx", "mm_integer.mtx", "mm_pattern.mtx", "mm_symmetric.mtx", "mm_upper_banner.mtx"]


def _stable_csr(n, row, col, val):
    """The reference's coo2csr ordering: stable by row (src/matrix.c:206-242)."""
    order = np.argsort(row, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, row.astype(np.int64) + 1, 1)
    return np.cumsum(ptr).astype(np.uint32), col[order], val[order]


def _python_parse(path):
    lines = open(path).read().splitlines()
    head = lines[0].split()
    field = head[3].lower()
    i = 1
    while lines[i].startswith("%") or not lines[i].strip():
        i += 1
    m, n, nz = map(int, lines[i].split())
    rows, cols, vals = [], [], []
    for ln in lines[i + 1:]:
        t = ln.split()
        if not t:
            continue
        rows.append(int(t[0]) - 1)
        cols.append(int(t[1]) - 1)
        vals.append(1.0 if field == "pattern" else float(t[2]))
    return m, n, np.array(rows, np.uint32), np.array(cols, np.uint32), np.array(vals)


@pytest.mark.parametrize("name", MM_NAMES)
def test_reader_matches_reference_loader(pkg, name):
    g = golden("mm_loader")
    c = pkg.read_mm(str(GOLDEN / name))
    assert (c["rows"], c["cols"], len(c["val"])) == (int(g[f"{name}:m"]), int(g[f"{name}:n"]), int(g[f"{name}:nz"]))
    ptr, col, val = _stable_csr(c["rows"], c["row"], c["col"], c["val"])
    assert np.array_equal(ptr, g[f"{name}:ptr"]) and np.array_equal(col, g[f"{name}:col"])
    assert np.array_equal(val, g[f"{name}:val"])
    assert (c["symmetry"] == "symmetric") == bool(int(g[f"{name}:symmetric"]))


def _random_file(path, n, nnz, seed, field="real", sym="general", scatter=True):
    rng = np.random.default_rng(seed)
    row = rng.integers(0, n, nnz)
    col = rng.integers(0, n, nnz)
    if sym != "general":
        row, col = np.maximum(row, col), np.minimum(row, col)
        if sym == "skew-symmetric":
            keep = row != col
            row, col = row[keep], col[keep]
    val = rng.standard_normal(len(row)) * 10.0 ** rng.uniform(-300, 300, len(row))
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {sym}\n% a comment\n%\n")
        f.write(f"{n} {n} {len(row)}\n")
        for r, c, v in zip(row, col, val):
            if field == "pattern":
                f.write(f"{r + 1} {c + 1}\n")
            elif field == "integer":
                f.write(f"{r + 1}  {c + 1}\t{int(v) % 100000 - 50000}\n")
            else:
                f.write(f"{r + 1} {c + 1} {v:.17g}\n" if scatter else f"{r + 1} {c + 1} {v!r}\n")
    return path


@pytest.mark.parametrize("field", ["real", "integer", "pattern"])
@pytest.mark.parametrize("threads", [1, 3, 16])
def test_reader_matches_python_parse(pkg, tmp_path, field, threads):
    path = _random_file(tmp_path / "r.mtx", 3000, 60000, seed=7, field=field)
    m, n, row, col, val = _python_parse(path)
    c = pkg.read_mm(str(path), threads=threads)
    assert (c["rows"], c["cols"]) == (m, n)
    assert np.array_equal(c["row"], row) and np.array_equal(c["col"], col)
    assert np.array_equal(c["val"].view(np.uint64), val.view(np.uint64))  # bit for bit


@pytest.mark.parametrize("sym,sign", [("symmetric", 1.0), ("skew-symmetric", -1.0)])
def test_symmetric_expansion(pkg, tmp_path, sym, sign):
    path = _random_file(tmp_path / "s.mtx", 500, 4000, seed=3, sym=sym)
    stored = pkg.read_mm(str(path))
    assert stored["symmetry"] == sym and not stored["expanded"]
    full = pkg.read_mm(str(path), expand_symmetric=True, threads=4)
    k = len(stored["val"])
    off = stored["row"] != stored["col"]
    assert full["expanded"] and len(full["val"]) == k + int(off.sum())
    assert np.array_equal(full["row"][:k], stored["row"]) and np.array_equal(full["val"][:k], stored["val"])
    assert np.array_equal(full["row"][k:], stored["col"][off]) and np.array_equal(full["col"][k:], stored["row"][off])
    assert np.array_equal(full["val"][k:], sign * stored["val"][off])


@pytest.mark.parametrize("text,what", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", "field"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n2 2 2\n", "entries"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n3 2 2\n", "index"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n2 2 x\n", "value"),
    ("not a matrix\n", "Matrix Market"),
])
def test_reader_rejects_bad_files(pkg, tmp_path, text, what):
    path = tmp_path / "bad.mtx"
    path.write_text(text)
    with pytest.raises(RuntimeError, match=what):
        pkg.read_mm(str(path))


def test_reader_missing_file(pkg, tmp_path):
    with pytest.raises(RuntimeError, match="cannot open"):
        pkg.read_mm(str(tmp_path / "none.mtx"))


def test_dropin_loader_uses_same_entries(pkg, lib, tmp_path):
    """csr_load_matrix (the reference's entry point, now parsing in parallel)
    gives the stable row order of the file's entries."""
    import ctypes as C

    path = _random_file(tmp_path / "d.mtx", 2000, 30000, seed=11)
    c = pkg.read_mm(str(path))
    ptr, col, val = _stable_csr(c["rows"], c["row"], c["col"], c["val"])
    m = pkg.CSR_Matrix()
    lib.csr_load_matrix(str(path).encode(), C.byref(m))
    n, nz = m.rows, m.nz
    got = (np.ctypeslib.as_array(m.ptr, shape=(n + 1,)).copy(), np.ctypeslib.as_array(m.col, shape=(nz,)).copy(),
           np.ctypeslib.as_array(m.val, shape=(nz,)).copy())
    lib.csr_free_matrix(C.byref(m))
    assert np.array_equal(got[0], ptr) and np.array_equal(got[1], col) and np.array_equal(got[2], val)
