"""Regenerate the golden vectors in this folder from the reference itself.

Run from the repository root where the reference sources are present:
    python tests/golden/make_golden.py [--ref-src <reference>/src]
It builds oracle/_ref/libref.so (the reference's own solver and loader compiled
single-rank through oracle/shim, see oracle/Makefile), runs it on small seeded
inputs and stores inputs and outputs as .npz, plus small Matrix Market files
with what the reference's loaders make of them.  The tests read only the
files written here; they never need the reference at run time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "oracle"))


def _workloads():
    spec = importlib.util.spec_from_file_location("hbicg_workloads_gen", ROOT / "hybrid-bicg_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def solver_cases(wl):
    """(name, csr, b, sigma, seed, tol, max_iter, variant, switching)"""
    cases = []
    a8 = wl.stencil_cd3d(8)
    b8 = np.full(a8.n, 1.0 / np.sqrt(a8.n))
    s6 = 0.01 * np.arange(6, dtype=np.float64)
    cases.append(("stencil8_seed0", a8, b8, s6, 0, 1e-10, 10000, "dynamic", True))
    cases.append(("stencil8_seed5", a8, b8, s6, 5, 1e-10, 10000, "dynamic", True))
    cases.append(("stencil8_seed5_static", a8, b8, s6, 5, 1e-10, 10000, "static", True))
    cases.append(("stencil8_seed5_normal", a8, b8, s6, 5, 1e-10, 10000, "normal", True))
    cases.append(("stencil8_maxiter5", a8, b8, s6, 0, 1e-10, 5, "dynamic", True))
    cases.append(("stencil8_single_shift", a8, b8, np.array([0.05]), 0, 1e-10, 10000, "dynamic", True))
    # two seed switches: irregular matrix, shifts in [-0.2, 1] (found by a seeded search)
    rng = np.random.default_rng(165)
    n = int(rng.integers(300, 1500))
    a_irr = wl.irregular_powerlaw(n, mean_len=8, max_len=60, seed=165)
    m = int(rng.integers(4, 10))
    sig = rng.uniform(-0.2, 1.0, m)
    b = rng.standard_normal(a_irr.n)
    seed = int(rng.integers(0, m))
    cases.append(("irregular_two_switches", a_irr, b, sig, seed, 1e-10, 3000, "dynamic", True))
    cases.append(("irregular_fixed_seed", a_irr, b, sig, seed, 1e-10, 3000, "dynamic", False))
    # two seed switches that survive 1e-14 relative perturbations of b (seeded
    # search); the case above is chaotic: its switch points move under rounding
    rng = np.random.default_rng(1060)
    a_r = wl.stencil_cd2d(int(rng.integers(8, 24)))
    m = int(rng.integers(4, 10))
    sig = rng.uniform(-0.5, 2.0, m)
    b = rng.standard_normal(a_r.n)
    seed = int(rng.integers(0, m))
    cases.append(("stencil2d_two_switches", a_r, b, sig, seed, 1e-10, 2000, "dynamic", True))
    a2 = wl.stencil_cd2d(12)
    rng2 = np.random.default_rng(7)
    b2 = rng2.standard_normal(a2.n)
    s2 = np.sort(rng2.uniform(1e-3, 1.0, 9))
    cases.append(("stencil2d_seed8", a2, b2, s2, 8, 1e-10, 10000, "dynamic", True))
    return cases


MM_FILES = {
    "mm_real_general.mtx": (
        "%%MatrixMarket matrix coordinate real general\n"
        "% a comment line\n"
        "%another comment\n"
        "4 4 9\n"
        "1 1 4.0\n3 1 -1.5\n2 2 5.25\n1 2 -1\n4 4 3e0\n2 3 -0.125\n3 3 6.0\n4 3 -2.0\n3 4 1.0E-1\n"),
    "mm_integer.mtx": (
        "%%MatrixMarket matrix coordinate integer general\n"
        "3 3 5\n"
        "1 1 7\n2 2 -3\n3 3 9\n3 1 2\n1 3 -4\n"),
    "mm_pattern.mtx": (
        "%%MatrixMarket matrix coordinate pattern general\n"
        "3 3 4\n"
        "1 1\n2 2\n3 3\n2 1\n"),
    "mm_symmetric.mtx": (
        "%%MatrixMarket matrix coordinate real symmetric\n"
        "3 3 4\n"
        "1 1 2.0\n2 1 -1.0\n2 2 2.0\n3 3 2.0\n"),
    "mm_upper_banner.mtx": (
        "%%MatrixMarket MATRIX Coordinate REAL General\n"
        "2 2 2\n"
        "2 2 1.5\n1 1 2.5\n"),
}


def mm_cases(lib):
    out = {}
    for name, text in MM_FILES.items():
        path = OUT / name
        path.write_text(text)
        code = C.create_string_buffer(5)
        mm, nn, nz = C.c_int(), C.c_int(), C.c_int()
        rc = lib.ref_read_header(str(path).encode(), code, C.byref(mm), C.byref(nn), C.byref(nz))
        n_out, nz_out = C.c_uint(), C.c_uint()
        sym = lib.ref_load_csr(str(path).encode(), C.byref(n_out), C.byref(nz_out), None, None, None)
        ptr = np.zeros(n_out.value + 1, dtype=np.uint32)
        col = np.zeros(nz_out.value, dtype=np.uint32)
        val = np.zeros(nz_out.value)
        lib.ref_load_csr(str(path).encode(), C.byref(n_out), C.byref(nz_out), ptr.ctypes.data_as(C.c_void_p),
                         col.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p))
        rec = {"header_rc": rc, "code": code.raw[:4].decode(), "m": mm.value, "n": nn.value, "nz": nz.value,
               "symmetric": sym, "ptr": ptr, "col": col, "val": val}
        if "real" in text.splitlines()[0].lower():
            # the row-block (MPI) loader reads values only for real files (src/matrix.c:321-331)
            lib.ref_load_block(str(path).encode(), C.byref(n_out), C.byref(nz_out), None, None, None, None)
            bptr = np.zeros(n_out.value + 1, dtype=np.uint32)
            bcol = np.zeros(nz_out.value, dtype=np.uint32)
            bval = np.zeros(nz_out.value)
            lib.ref_load_block(str(path).encode(), C.byref(n_out), C.byref(nz_out), bptr.ctypes.data_as(C.c_void_p),
                               bcol.ctypes.data_as(C.c_void_p), bval.ctypes.data_as(C.c_void_p), None)
            rec.update(block_ptr=bptr, block_col=bcol, block_val=bval)
        out[name] = rec
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=None)
    args = ap.parse_args()
    import oracle as O
    if args.ref_src:
        O.REF_SRC = Path(args.ref_src)
    O.build(ref=True)
    wl = _workloads()
    for (name, a, b, sigma, seed, tol, maxit, variant, switching) in solver_cases(wl):
        res = O.ref_solve(a, b, sigma, seed=seed, tol=tol, max_iter=maxit, variant=variant, switching=switching)
        sw = np.array(res.switches, dtype=np.int64).reshape(-1, 2)
        np.savez_compressed(OUT / f"{name}.npz", ptr=a.ptr, col=a.col, val=a.val, b=b, sigma=sigma, seed=seed,
                            tol=tol, max_iter=maxit, variant=variant, switching=switching, k=res.k, x=res.x,
                            r=res.r, switches=sw)
        print(f"{name}: n={a.n} m={len(sigma)} k={res.k} switches={res.switches}")
    # SpMV through the reference's serial product (src/matrix.c:498-516)
    a = wl.irregular_powerlaw(1500, mean_len=12, max_len=400, seed=11)
    x = np.random.default_rng(12).standard_normal(a.n)
    np.savez_compressed(OUT / "spmv_irregular.npz", ptr=a.ptr, col=a.col, val=a.val, x=x, y=O.ref_spmv(a, x))
    lib = O.ref_lib()
    lib.ref_read_header.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ref_load_csr.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ref_load_block.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]
    mm = mm_cases(lib)
    flat = {}
    for name, rec in mm.items():
        for key, v in rec.items():
            flat[f"{name}:{key}"] = np.asarray(v)
    np.savez_compressed(OUT / "mm_loader.npz", **flat)
    print("mm files:", ", ".join(mm))




def convergence_profile(name: str = "c2") -> None:
    """Convergence profile of a named workload from the oracle (the reference's
    algorithm): the seed system alone is solved to convergence, then every
    shift's convergence iteration is replayed from the seed's scalar history
    (no switching: the seed is the smallest shift and converges last).  The
    benchmark's CPU baseline costs a full solve from this profile and a timed
    bounded sample, so it does not need the hours-long full CPU solve."""
    import oracle as O
    import time

    O.build(ref=False)
    wl = _workloads()
    f = wl.family(name)
    t0 = time.perf_counter()
    seed_run = O.solve(f.a, f.b, f.sigma[f.seed:f.seed + 1], seed=0, tol=f.tol, max_iter=f.max_iter)
    secs = time.perf_counter() - t0
    conv, act = O.shift_profile(seed_run.hist, f.sigma, f.seed, f.tol, float(f.b @ f.b))
    out = {"workload": name, "k": int(seed_run.k), "conv_k": [int(c) for c in conv],
           "active_per_iter": [int(a) for a in act[:seed_run.k]], "shift_updates": int(act.sum()),
           "oracle_seconds": secs}
    import json

    (OUT / f"{name}_profile.json").write_text(json.dumps(out) + "\n")
    print(f"{name}: k={seed_run.k} shift updates={int(act.sum())} ({secs:.0f} s)")


DIGEST_SAMPLES = 4096


def digest_indices(n: int, count: int = DIGEST_SAMPLES) -> np.ndarray:
    """Rows sampled by a solution digest: seeded, sorted, first and last row included."""
    idx = np.random.default_rng(20261204).choice(n, size=min(count, n) - 2, replace=False)
    return np.unique(np.concatenate([idx, [0, n - 1]])).astype(np.int64)


def solution_digest(name: str = "c2", scale: int | None = None) -> None:
    """Digest of the reference's own full solve of a named workload (at its
    full size, or at grid side `scale`: file <name>_<scale>_digest.npz).

    The reference (oracle/_ref/libref.so, its sources compiled single-rank) runs
    the whole family to convergence with the workload's tolerance; the digest
    keeps what a test needs to compare another solver's 64 solutions with it
    without the 8.6 GB of x: k, the switch sequence, every shift's norm, sum and
    true residual, and every shift's values at DIGEST_SAMPLES seeded rows."""
    import oracle as O
    import time

    O.build(ref=True)
    wl = _workloads()
    f = wl.family(name, scale)
    t0 = time.perf_counter()
    res = O.ref_solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=f.max_iter, variant="dynamic")
    secs = time.perf_counter() - t0
    idx = digest_indices(f.a.n)
    tr = O.true_residuals(f.a, res.x, f.b, f.sigma)
    sw = np.array(res.switches, dtype=np.int64).reshape(-1, 2)
    tag = name if scale is None else f"{name}_{scale}"
    np.savez_compressed(OUT / f"{tag}_digest.npz", k=res.k, switches=sw, sigma=f.sigma, idx=idx,
                        x_at=res.x[:, idx], norm=np.linalg.norm(res.x, axis=1), sum=res.x.sum(axis=1),
                        true_residual=tr, r_at=res.r[idx], seconds=secs)
    print(f"{tag}: k={res.k} switches={res.switches} max true residual={tr.max():.3e} ({secs:.0f} s)")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--profile":
        convergence_profile(sys.argv[2])
    elif len(sys.argv) > 2 and sys.argv[1] == "--digest":
        solution_digest(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else None)
    else:
        main()
