"""A C program that calls the library the way the reference's driver calls
its solver (src/main.c:88-151): it includes only include/*.h, links only
libhbicg.so and calls MPI_csr_load_matrix_block and shifted_lopbicg_*.  The
build is checked without a GPU; the run is checked on the GPU against the
oracle (the reference's algorithm) on the same matrix file, with the
reference's compile-time EPS (1e-12) and MAX_ITER (2000)."""
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
