"""C programs linked against the library, including only include/*.h and
linking only libhbicg.so: one calls it the way the reference's driver calls
its solver (src/main.c:88-151: MPI_csr_load_matrix_block and
shifted_lopbicg_*, with the reference's compile-time EPS 1e-12 and MAX_ITER
2000); the other solves several Matrix Market files in one
hbicg_batch_solve_opts call.  The builds are checked without a GPU; the runs
on the GPU against the oracle (the reference's algorithm) on the same
matrices."""
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = ROOT / "tests" / "c_driver" / "reference_main.c"


def build_driver(pkg, out_dir):
    exe = out_dir / "reference_main"
    libdir = pkg.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC),
                    f"-L{libdir}", "-lhbicg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def test_reference_style_driver_builds_and_links(lib, pkg, tmp_path):
    exe = build_driver(pkg, tmp_path)
    ldd = subprocess.run(["ldd", str(exe)], capture_output=True, text=True).stdout
    assert "libhbicg.so" in ldd


@pytest.mark.gpu
@pytest.mark.parametrize("variant,seed", [("dynamic", 0), ("static", 3), ("normal", 7)])
def test_reference_style_driver_matches_oracle(cuda, pkg, oracle, tmp_path, variant, seed):
    a = pkg.workloads.stencil_cd3d(10, 9, 8)
    mtx = tmp_path / "a.mtx"
    pkg.workloads.write_matrix_market(str(mtx), a)
    m = 8
    exe = build_driver(pkg, tmp_path)
    out = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(mtx), str(m), str(seed), variant, str(out)], capture_output=True, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    raw = out.read_bytes()
    k, rows, sl = np.frombuffer(raw[:12], dtype=np.int32)
    assert rows == a.n and sl == m
    body = np.frombuffer(raw[12:], dtype=np.float64)
    x = body[:m * rows].reshape(m, rows)
    r = body[m * rows:]
    # the driver's inputs, restated: sigma_i = (i + 1) (0.01 / m), b = 1
    sigma = (np.arange(m) + 1) * (0.01 / m)
    b = np.ones(a.n)
    want = oracle.solve(a, b, sigma, seed=seed, tol=1e-12, max_iter=2000)
    assert abs(int(k) - want.k) <= max(1, int(0.02 * want.k)), (k, want.k)
    err = np.max(np.abs(x - want.x)) / np.max(np.abs(want.x))
    assert err < 1e-8, err
    res = oracle.true_residuals(a, x, b, sigma)
    res_ref = oracle.true_residuals(a, want.x, b, sigma)
    assert np.all(res <= np.maximum(1e-12 * 1.001, 1.1 * res_ref)), (res, res_ref)
    assert np.all(np.isfinite(r))


BATCH_SRC = ROOT / "tests" / "c_driver" / "batch_main.c"


def build_batch_driver(pkg, out_dir):
    exe = out_dir / "batch_main"
    libdir = pkg.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(BATCH_SRC),
                    f"-L{libdir}", "-lhbicg", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def test_batch_driver_builds_and_links(lib, pkg, tmp_path):
    exe = build_batch_driver(pkg, tmp_path)
    assert "libhbicg.so" in subprocess.run(["ldd", str(exe)], capture_output=True, text=True).stdout


@pytest.mark.gpu
def test_batch_driver_matches_oracle(cuda, pkg, oracle, tmp_path):
    """A C program calls hbicg_batch_solve_opts on three Matrix Market files
    (the small families go to the shared persistent launch): every family
    converges and its solutions match the oracle's (the reference's
    algorithm) to 1e-8."""
    mats = [pkg.workloads.stencil_cd3d(9, 8, 7), pkg.workloads.stencil_cd2d(30), pkg.workloads.stencil_cd3d(12)]
    paths = []
    for i, a in enumerate(mats):
        p = tmp_path / f"a{i}.mtx"
        pkg.workloads.write_matrix_market(str(p), a)
        paths.append(str(p))
    m = 6
    exe = build_batch_driver(pkg, tmp_path)
    out = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(m), str(out)] + paths, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    raw = out.read_bytes()
    off = 0
    sigma = (np.arange(m) + 1) * (0.01 / m)
    for a in mats:
        status, k, rows = np.frombuffer(raw[off:off + 12], dtype=np.int32)
        off += 12
        x = np.frombuffer(raw[off:off + 8 * m * rows], dtype=np.float64).reshape(m, rows)
        off += 8 * m * rows
        assert status == 0 and rows == a.n
        want = oracle.solve(a, np.ones(a.n), sigma, seed=0, tol=1e-10, max_iter=5000)
        assert np.max(np.abs(x - want.x)) < 1e-8 * np.max(np.abs(want.x))
