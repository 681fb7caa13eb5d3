"""The C-ABI library without a GPU: it loads, exports every function the
headers in include/ declare, and its host-side loaders and helpers match the
reference (golden outputs of the reference's own loaders)."""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}()]*(?:\([^()]*\)[^;{}()]*)*)\)\s*;", text):
            name = m.group(1)
            if name in {"if", "while", "for", "return", "sizeof"}:
                continue
            names.add(name)
    return names


def test_headers_declare_the_reference_surface():
    names = declared_functions()
    for fn in ["shifted_lopbicg_dynamic", "shifted_lopbicg_static", "shifted_lopbicg_normal", "coo2csr",
               "csr_load_matrix", "MPI_csr_load_matrix_block", "mult", "csr_shift_diagonal", "my_daxpy",
               "my_ddot", "mm_read_banner", "mm_read_mtx_crd_size", "hbicg_solve"]:
        assert fn in names, fn


def test_library_exports_every_declared_symbol(lib, pkg):
    out = subprocess.run(["nm", "-D", "--defined-only", str(pkg.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(declared_functions() - exported)
    assert not missing, missing
    for name in declared_functions():
        getattr(lib, name)


def test_headers_compile_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "solver.h"\n#include "hbicg.h"\nint main(void){CSR_Matrix a; csr_init_matrix(&a);'
                   'return (int)sizeof(INFO_Matrix) > 0 ? 0 : 1;}\n')
    for cc, extra in (("gcc", ["-std=c99"]), ("g++", ["-x", "c++"])):
        subprocess.run([cc, *extra, "-fsyntax-only", f"-I{ROOT / 'include'}", str(src)], check=True)


def test_struct_layouts_match_reference(pkg):
    # src/matrix.h:10-33 with 64-bit pointers
    assert C.sizeof(pkg.CSR_Matrix) == 3 * 8 + 3 * 4 + 4
    assert pkg.CSR_Matrix.nz.offset == 24 and pkg.CSR_Matrix.cols.offset == 32
    assert pkg.INFO_Matrix.code.offset == 12 and pkg.INFO_Matrix.recvcounts.offset == 16


MM_NAMES = ["mm_real_general.mtx", "mm_integer.mtx", "mm_pattern.mtx", "mm_symmetric.mtx", "mm_upper_banner.mtx"]


@pytest.mark.parametrize("name", MM_NAMES)
def test_banner_and_size_match_reference(lib, name):
    g = golden("mm_loader")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    f = libc.fopen(str(GOLDEN / name).encode(), b"r")
    code = (C.c_char * 4)()
    rc = lib.mm_read_banner(f, C.cast(code, C.c_void_p))
    mm, nn, nz = C.c_int(), C.c_int(), C.c_int()
    if rc == 0:
        rc = lib.mm_read_mtx_crd_size(f, C.byref(mm), C.byref(nn), C.byref(nz))
    libc.fclose(f)
    assert rc == int(g[f"{name}:header_rc"])
    assert bytes(code).decode() == str(g[f"{name}:code"])
    assert (mm.value, nn.value, nz.value) == (int(g[f"{name}:m"]), int(g[f"{name}:n"]), int(g[f"{name}:nz"]))


@pytest.mark.parametrize("name", MM_NAMES)
def test_serial_loader_matches_reference(lib, pkg, name):
    g = golden("mm_loader")
    m = pkg.CSR_Matrix()
    sym = lib.csr_load_matrix(str(GOLDEN / name).encode(), C.byref(m))
    n, nz = m.rows, m.nz
    ptr = np.ctypeslib.as_array(m.ptr, shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(m.col, shape=(nz,)).copy()
    val = np.ctypeslib.as_array(m.val, shape=(nz,)).copy()
    lib.csr_free_matrix(C.byref(m))
    assert sym == int(g[f"{name}:symmetric"])
    assert np.array_equal(ptr, g[f"{name}:ptr"]) and np.array_equal(col, g[f"{name}:col"])
    assert np.array_equal(val, g[f"{name}:val"])


@pytest.mark.parametrize("name", [n for n in MM_NAMES if n != "mm_integer.mtx" and n != "mm_pattern.mtx"])
def test_row_block_loader_matches_reference(pkg, name):
    g = golden("mm_loader")
    a, code, offd_nz = pkg.load_matrix_market(str(GOLDEN / name))
    assert offd_nz == 0
    assert code == str(g[f"{name}:code"])
    assert np.array_equal(a.ptr, g[f"{name}:block_ptr"]) and np.array_equal(a.col, g[f"{name}:block_col"])
    assert np.array_equal(a.val, g[f"{name}:block_val"])


def test_row_block_loader_reads_integer_and_pattern_values(pkg):
    # the reference leaves these values unset (src/matrix.c:316-331); here they are read
    a, code, _ = pkg.load_matrix_market(str(GOLDEN / "mm_integer.mtx"))
    assert code == "MCIG" and np.array_equal(a.val, golden("mm_loader")["mm_integer.mtx:val"])
    a, code, _ = pkg.load_matrix_market(str(GOLDEN / "mm_pattern.mtx"))
    assert code == "MCPG" and np.all(a.val == 1.0)


def test_matrix_market_round_trip(pkg, tmp_path):
    a = pkg.workloads.stencil_cd3d(6, 5, 4)
    path = tmp_path / "s.mtx"
    pkg.workloads.write_matrix_market(str(path), a, comment="round trip")
    b, code, _ = pkg.load_matrix_market(str(path))
    assert code == "MCRG"
    assert np.array_equal(a.ptr, b.ptr) and np.array_equal(a.col, b.col) and np.array_equal(a.val, b.val)


def test_coo_sorts_are_stable(lib):
    rng = np.random.default_rng(0)
    nz = 500
    rows = rng.integers(0, 20, nz).astype(np.uint32)
    cols = np.arange(nz, dtype=np.uint32)
    vals = rng.standard_normal(nz)
    order = np.argsort(rows, kind="stable")
    A, A2, A3 = rows.copy(), cols.copy(), vals.copy()
    B, B2, B3 = np.zeros_like(A), np.zeros_like(A2), np.zeros_like(A3)
    pu = C.POINTER(C.c_uint)
    pd = C.POINTER(C.c_double)
    lib.coo_merge_sort.argtypes = [pu, pu, pd, pu, pu, pd, C.c_int, C.c_int]
    lib.coo_merge_sort(A.ctypes.data_as(pu), A2.ctypes.data_as(pu), A3.ctypes.data_as(pd), B.ctypes.data_as(pu),
                       B2.ctypes.data_as(pu), B3.ctypes.data_as(pd), 0, nz - 1)
    assert np.array_equal(A, rows[order]) and np.array_equal(A2, cols[order]) and np.array_equal(A3, vals[order])


def test_host_vector_helpers(lib):
    pd = C.POINTER(C.c_double)
    lib.my_daxpy.argtypes = [C.c_int, C.c_double, pd, pd]
    lib.my_ddot.argtypes = [C.c_int, pd, pd]
    lib.my_ddot.restype = C.c_double
    x = np.arange(5.0)
    y = np.ones(5)
    lib.my_daxpy(5, 2.0, x.ctypes.data_as(pd), y.ctypes.data_as(pd))
    assert np.array_equal(y, 1 + 2 * x)
    assert lib.my_ddot(5, x.ctypes.data_as(pd), y.ctypes.data_as(pd)) == float(np.dot(x, y))


def test_noalloc_wrapper_rejects_bad_tensors(pkg):
    """The Python wrapper of hbicg_true_residuals_noalloc refuses tensors the
    kernels would read or write past, before any call into the library (host
    tensors are enough to check the shape, dtype and layout rules)."""
    torch = pytest.importorskip("torch")
    n, m = 10, 3
    f64 = dict(dtype=torch.float64)
    ok = dict(x=torch.zeros(m, n, **f64), b=torch.zeros(n, **f64), sigma=torch.zeros(m, **f64),
              res=torch.zeros(m, **f64))
    bad_cases = [
        dict(x=torch.zeros(m, n, dtype=torch.float32)),
        dict(x=torch.zeros(m * n, **f64)),                    # one-dimensional x
        dict(x=torch.zeros(m - 1, n, **f64)),                 # fewer rows than shifts
        dict(x=torch.zeros(m, n - 1, **f64)),                 # rows shorter than n
        dict(x=torch.zeros(n, m, **f64).t()),                 # inner stride m
        dict(b=torch.zeros(n - 1, **f64)),
        dict(res=torch.zeros(m - 1, **f64)),
        dict(sigma=torch.zeros(m, 1, **f64)),
        dict(b=torch.zeros(2 * n, **f64)[::2]),               # strided b
        dict(res=[0.0] * m),
    ]
    for bad in bad_cases:
        args = {**ok, **bad}
        with pytest.raises(ValueError):
            pkg._check_noalloc_args(n, args["x"], args["b"], args["sigma"], args["res"])
    # well-formed host tensors fail only on the device rule
    with pytest.raises(ValueError, match="CUDA"):
        pkg._check_noalloc_args(n, ok["x"], ok["b"], ok["sigma"], ok["res"])
    # wider rows (a leading dimension above n) are allowed
    wide = torch.zeros(m, n + 6, **f64)
    with pytest.raises(ValueError, match="CUDA"):
        pkg._check_noalloc_args(n, wide, ok["b"], ok["sigma"], ok["res"])


def test_batch_options_and_graph_modes_on_the_host(pkg):
    """The batch options' defaults (hbicg_batch_opts_default) and the Python
    mapping of the graph and shared-launch modes onto the C parameters."""
    o = pkg.BatchOpts()
    pkg.lib().hbicg_batch_opts_default(C.byref(o))
    assert (o.workers, o.persistent, o.persistent_ctas, o.autotune_cache) == (8, 1, 0, None)
    assert pkg.params().use_graph == 1
    assert [pkg.params(use_graph=v).use_graph for v in (False, True, "loop", "persistent")] == [0, 1, 2, 3]
    p = pkg.params()
    assert (p.basis_block, p.refine, p.shift_mode) == (0, 1, 0)
