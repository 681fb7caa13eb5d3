"""TEST INFRASTRUCTURE — the oracle.

ctypes access to the two CPU checkers built by oracle/Makefile:
  * liboracle.so      — the C restatement (hbicg_oracle.c) of the reference's
                        shifted BiCGStab with seed switching and its CSR SpMV;
  * _ref/libref.so    — the reference's own sources compiled single-rank through
                        oracle/shim (exists only where the reference is present).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs use this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_SRC = Path(os.environ.get("HBICG_REF_SRC", "/root/reference/src"))

_PD = C.POINTER(C.c_double)
_PU = C.POINTER(C.c_uint)
_PI = C.POINTER(C.c_int)


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """make the restatement; also the reference build when its sources exist."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True, stdout=out)
    if ref is None:
        ref = REF_SRC.is_dir()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True, stdout=out)


class _Opts(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("switching", C.c_int), ("schedule", C.c_int)]


class _Trace(C.Structure):
    _fields_ = [("sw_k", _PI), ("sw_seed", _PI), ("sw_cap", C.c_int), ("n_sw", C.c_int), ("act", _PI),
                ("act_cap", C.c_int), ("conv_k", _PI), ("final_seed", C.c_int), ("a_hist", _PD), ("b_hist", _PD),
                ("w_hist", _PD), ("rr_hist", _PD), ("hist_cap", C.c_int), ("t_iter", _PD), ("t_cap", C.c_int)]


@dataclass
class OracleResult:
    k: int                 # the reference's return value (iterations + 1 on convergence)
    x: np.ndarray          # (m, n)
    r: np.ndarray          # final seed residual (the reference's r_loc on exit)
    switches: list         # [(k, new_seed), ...]
    act: np.ndarray | None = None      # active non-seed shifts per iteration (index k)
    conv_k: np.ndarray | None = None   # iteration at which each shift converged
    final_seed: int | None = None
    hist: dict | None = None           # seed alpha/beta/omega and (r,r) per iteration


def _p(a, t):
    return a.ctypes.data_as(t)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            build(ref=False)
        _lib = C.CDLL(str(path))
        _lib.hbo_shifted_bicgstab.restype = C.c_int
        _lib.hbo_shifted_bicgstab.argtypes = [C.c_uint, _PU, _PU, _PD, _PD, _PD, _PD, C.c_int, C.c_int,
                                              C.POINTER(_Opts), C.POINTER(_Trace)]
        _lib.hbo_spmv.argtypes = [C.c_uint, _PU, _PU, _PD, _PD, _PD]
        _lib.hbo_spmv_fma.argtypes = [C.c_uint, _PU, _PU, _PD, _PD, _PD]
        _lib.hbo_true_residuals.argtypes = [C.c_uint, _PU, _PU, _PD, _PD, _PD, _PD, C.c_int, _PD]
    return _lib


def ref_available() -> bool:
    return (HERE / "_ref" / "libref.so").exists()


def ref_lib():
    global _ref
    if _ref is None:
        path = HERE / "_ref" / "libref.so"
        if not path.exists():
            raise FileNotFoundError("oracle/_ref/libref.so is not built (the reference sources are absent)")
        _ref = C.CDLL(str(path))
        _ref.ref_solve.restype = C.c_int
        _ref.ref_solve.argtypes = [C.c_int, C.c_uint, _PU, _PU, _PD, _PD, _PD, _PD, C.c_int, C.c_int, C.c_double,
                                   C.c_int, _PI, _PI, C.c_int, _PI]
        _ref.ref_mult.argtypes = [C.c_uint, _PU, _PU, _PD, _PD, _PD]
    return _ref


def _csr(a):
    ptr = np.ascontiguousarray(a.ptr, dtype=np.uint32)
    col = np.ascontiguousarray(a.col, dtype=np.uint32)
    val = np.ascontiguousarray(a.val, dtype=np.float64)
    return ptr, col, val


SCHEDULES = {"dynamic": 0, "static": 1, "normal": 2}


def solve(a, b, sigma, seed=0, tol=1e-12, max_iter=2000, switching=True, schedule="dynamic") -> OracleResult:
    """The C restatement; same contract as the reference's shifted_lopbicg_*."""
    ptr, col, val = _csr(a)
    n, m = a.n, len(sigma)
    x = np.zeros((m, n))
    r = np.ascontiguousarray(b, dtype=np.float64).copy()
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    cap = max(m, 1) + 4
    swk = np.zeros(cap, dtype=np.int32)
    sws = np.zeros(cap, dtype=np.int32)
    act = np.zeros(max_iter + 2, dtype=np.int32)
    conv = np.zeros(max(m, 1), dtype=np.int32)
    hist = {key: np.zeros(max_iter + 2) for key in ("alpha", "beta", "omega", "rr", "t")}
    tr = _Trace(_p(swk, _PI), _p(sws, _PI), cap, 0, _p(act, _PI), act.shape[0], _p(conv, _PI), 0,
                _p(hist["alpha"], _PD), _p(hist["beta"], _PD), _p(hist["omega"], _PD), _p(hist["rr"], _PD),
                max_iter + 2, _p(hist["t"], _PD), max_iter + 2)
    opts = _Opts(float(tol), int(max_iter), 1 if switching else 0, SCHEDULES[schedule])
    k = lib().hbo_shifted_bicgstab(n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(x, _PD), _p(r, _PD),
                                   _p(sig, _PD), m, int(seed), C.byref(opts), C.byref(tr))
    sw = [(int(swk[i]), int(sws[i])) for i in range(min(tr.n_sw, cap))]
    hist = {key: v[:k].copy() for key, v in hist.items()}
    return OracleResult(k, x, r, sw, act[:k + 1].copy(), conv[:m].copy(), tr.final_seed, hist)


def shift_profile(hist, sigma, seed, tol, bb):
    """Replay the shift recurrences of src/solver_dynamic.c:243-253 from a seed's
    scalar history (no switching): the iteration at which every shift meets the
    convergence test (:294) and the number of non-seed shifts each iteration
    updates.  Used to cost a full multi-shift solve from a seed-only run."""
    a, b, w, rr = hist["alpha"], hist["beta"], hist["omega"], hist["rr"]
    kend = len(a)
    sig = np.asarray(sigma, dtype=np.float64)
    d = sig[seed] - sig
    m = len(sig)
    eta = np.zeros(m)
    zeta = np.ones(m)
    pi_prev = np.ones(m)
    conv = np.zeros(m, dtype=np.int64)
    act = np.zeros(kend + 1, dtype=np.int64)
    thr = tol * tol * bb
    for k in range(1, kend):
        running = conv == 0
        act[k] = int(running.sum()) - int(running[seed])
        c_prev = (b[k - 1] / a[k - 1]) * a[k]
        eta = c_prev * eta - d * a[k] * pi_prev
        pi = eta + pi_prev
        zeta = (1.0 - w[k] * d) * zeta
        fac = np.abs(1.0 / (zeta * pi))
        fac[seed] = 1.0
        newly = running & (fac * fac * rr[k] <= thr)
        conv[newly] = k
        pi_prev = pi
    return conv, act


def ref_solve(a, b, sigma, seed=0, tol=1e-12, max_iter=2000, variant="dynamic", switching=True) -> OracleResult:
    """The reference's own solver (oracle/_ref); variant in dynamic/static/normal."""
    v = {"dynamic": 0, "static": 1, "normal": 2}[variant]
    if not switching:
        if variant != "dynamic":
            raise ValueError("the fixed-seed reference build exists for the dynamic variant only")
        v = 3
    ptr, col, val = _csr(a)
    n, m = a.n, len(sigma)
    x = np.zeros((m, n))
    r = np.ascontiguousarray(b, dtype=np.float64).copy()
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    cap = max(m, 1) + 4
    swk = np.zeros(cap, dtype=np.int32)
    sws = np.zeros(cap, dtype=np.int32)
    nlog = C.c_int(0)
    k = ref_lib().ref_solve(v, n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(x, _PD), _p(r, _PD), _p(sig, _PD),
                            m, int(seed), float(tol), int(max_iter), _p(swk, _PI), _p(sws, _PI), cap, C.byref(nlog))
    sw = [(int(swk[i]), int(sws[i])) for i in range(min(nlog.value, cap))]
    return OracleResult(k, x, r, sw)


def spmv(a, x) -> np.ndarray:
    ptr, col, val = _csr(a)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.n)
    lib().hbo_spmv(a.n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(xx, _PD), _p(y, _PD))
    return y


def spmv_fma(a, x) -> np.ndarray:
    """Row sums as fused multiply-adds in stored order (the GPU kernel's order)."""
    ptr, col, val = _csr(a)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.n)
    lib().hbo_spmv_fma(a.n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(xx, _PD), _p(y, _PD))
    return y


def ref_spmv(a, x) -> np.ndarray:
    ptr, col, val = _csr(a)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.n)
    ref_lib().ref_mult(a.n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(xx, _PD), _p(y, _PD))
    return y


def true_residuals(a, x, b, sigma) -> np.ndarray:
    """||b - (A + sigma_j I) x_j|| / ||b|| for every shift."""
    ptr, col, val = _csr(a)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    out = np.zeros(len(sigma))
    lib().hbo_true_residuals(a.n, _p(ptr, _PU), _p(col, _PU), _p(val, _PD), _p(xx, _PD), _p(bb, _PD),
                             _p(sig, _PD), len(sigma), _p(out, _PD))
    return out
