"""Python binding of the GB300 shifted BiCGStab solver (libhbicg.so).

A thin ctypes layer over the C ABI in include/: the reference's drop-in entry
points (shifted_lopbicg_{dynamic,static,normal}, src/solver.h:33-35; the
matrix.h loaders and products) and the extended API (include/hbicg.h).  Host
arrays are numpy; device arrays are torch CUDA tensors (PyTorch is used only
for device memory and streams).  There is no CPU path: every call that
computes goes through the CUDA library, and loading fails loudly when it has
not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import workloads  # noqa: F401  (re-exported)

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libhbicg.so"
INCLUDE = HERE.parent / "include"

_PD = C.POINTER(C.c_double)
_PU = C.POINTER(C.c_uint)
_PI = C.POINTER(C.c_int)

HOST, DEVICE = 0, 1
FORMS = {"plain": 0, "fused": 1}
SHIFT_MODES = {"auto": 0, "incremental": 1, "deferred": 2}
FLUSH_MODES = {"auto": 0, "fp64": 1, "tensor": 2}
STATUS = {0: "ok", 1: "not square", 2: "no diagonal", 3: "breakdown", 4: "max_iter", 5: "cuda", 6: "timeout",
          7: "argument", 8: "out of memory", 9: "io"}


class HbicgError(RuntimeError):
    pass


def build(jobs: int | None = None, quiet: bool = True) -> Path:
    """Compile libhbicg.so for sm_103a (nvcc + gcc, no cmake)."""
    jobs = jobs or max(2, os.cpu_count() or 2)
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-j", str(jobs), "-C", str(HERE / "csrc")], check=True, stdout=out)
    return LIB_PATH


# ---------------------------------------------------------------- ctypes types
class COO_Matrix(C.Structure):
    """src/matrix.h:11-18"""
    _fields_ = [("val", _PD), ("row", _PU), ("col", _PU), ("nz", C.c_uint), ("rows", C.c_uint), ("cols", C.c_uint)]


class CSR_Matrix(C.Structure):
    """src/matrix.h:19-26"""
    _fields_ = [("val", _PD), ("col", _PU), ("ptr", _PU), ("nz", C.c_uint), ("rows", C.c_uint), ("cols", C.c_uint)]


class INFO_Matrix(C.Structure):
    """src/matrix.h:28-33 without MPI types"""
    _fields_ = [("nz", C.c_uint), ("rows", C.c_uint), ("cols", C.c_uint), ("code", C.c_char * 4),
                ("recvcounts", _PI), ("displs", _PI)]


class Params(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("switching", C.c_int), ("form", C.c_int),
                ("shift_mode", C.c_int), ("use_graph", C.c_int), ("graph_chunk", C.c_int),
                ("basis_mem_frac", C.c_double), ("true_residuals", C.c_int), ("basis_block", C.c_int),
                ("flush_mode", C.c_int), ("refine", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("k", C.c_int), ("status", C.c_int), ("n_switches", C.c_int), ("final_seed", C.c_int),
                ("shift_mode", C.c_int), ("basis_flushes", C.c_int), ("launches", C.c_int),
                ("refined_shifts", C.c_int),
                ("solve_ms", C.c_double), ("flush_ms", C.c_double), ("max_true_residual", C.c_double),
                ("bytes_algorithmic", C.c_double), ("flush_bytes", C.c_double),
                ("switch_k", _PI), ("switch_seed", _PI), ("conv_k", _PI), ("active_per_iter", _PI),
                ("true_residual", _PD), ("seed_alpha", _PD), ("seed_beta", _PD), ("seed_omega", _PD),
                ("seed_rr", _PD)]


class Coo(C.Structure):
    _fields_ = [("rows", C.c_uint), ("cols", C.c_uint), ("nnz", C.c_ulonglong), ("field", C.c_int),
                ("symmetry", C.c_int), ("expanded", C.c_int), ("row", _PU), ("col", _PU), ("val", _PD)]


class Family(C.Structure):
    """hbicg_family (include/hbicg.h)"""
    _fields_ = [("n", C.c_uint), ("nnz", C.c_uint), ("ptr", _PU), ("col", _PU), ("val", _PD), ("b", _PD),
                ("sigma", _PD), ("m", C.c_int), ("seed", C.c_int), ("autotune", C.c_int), ("x", _PD), ("r", _PD),
                ("true_residual", _PD), ("status", C.c_int), ("k", C.c_int), ("n_switches", C.c_int),
                ("final_seed", C.c_int), ("spmv_format", C.c_int), ("solve_ms", C.c_double),
                ("wall_ms", C.c_double), ("max_true_residual", C.c_double)]


class BatchOpts(C.Structure):
    """hbicg_batch_opts (include/hbicg.h)"""
    _fields_ = [("workers", C.c_int), ("persistent", C.c_int), ("persistent_ctas", C.c_int),
                ("autotune_cache", C.c_char_p)]


_lib = None


def lib() -> C.CDLL:
    """Load libhbicg.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise HbicgError(f"{LIB_PATH} is not built: call build() (needs nvcc); there is no CPU fallback")
    L = C.CDLL(str(LIB_PATH))
    sig = {
        "hbicg_params_default": (None, [C.POINTER(Params)]),
        "hbicg_status_string": (C.c_char_p, [C.c_int]),
        "hbicg_last_message": (C.c_char_p, []),
        "hbicg_context_create": (C.c_int, [C.POINTER(C.c_void_p)]),
        "hbicg_context_destroy": (None, [C.c_void_p]),
        "hbicg_context_stream": (C.c_void_p, [C.c_void_p]),
        "hbicg_matrix_create": (C.c_int, [C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                          C.POINTER(C.c_void_p)]),
        "hbicg_matrix_destroy": (None, [C.c_void_p]),
        "hbicg_matrix_rows": (C.c_uint, [C.c_void_p]),
        "hbicg_matrix_nnz": (C.c_ulonglong, [C.c_void_p]),
        "hbicg_mm_read": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(Coo)]),
        "hbicg_coo_free": (None, [C.POINTER(Coo)]),
        "hbicg_matrix_from_coo": (C.c_int, [C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_int, C.POINTER(C.c_void_p)]),
        "hbicg_matrix_load_mm": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
        "hbicg_matrix_get_csr": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
        "hbicg_matrix_format": (C.c_int, [C.c_void_p]),
        "hbicg_release": (None, []),
        "hbicg_matrix_transpose": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
        "hbicg_adjoint_gradients": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_ulonglong, C.c_void_p,
                                              C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "hbicg_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                    C.c_void_p, C.POINTER(Params), C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "hbicg_matrix_set_format": (C.c_int, [C.c_void_p, C.c_int]),
        "hbicg_matrix_autotune": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]),
        "hbicg_batch_solve": (C.c_int, [C.POINTER(Family), C.c_int, C.POINTER(Params), C.c_int, C.c_char_p,
                                        C.POINTER(C.c_double)]),
        "hbicg_batch_opts_default": (None, [C.POINTER(BatchOpts)]),
        "hbicg_batch_solve_opts": (C.c_int, [C.POINTER(Family), C.c_int, C.POINTER(Params), C.POINTER(BatchOpts),
                                             C.POINTER(C.c_double)]),
        "hbicg_matrix_spmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]),
        "hbicg_matrix_time_spmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                             C.POINTER(C.c_double)]),
        "hbicg_solver_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(Params), C.POINTER(C.c_void_p)]),
        "hbicg_solver_destroy": (None, [C.c_void_p]),
        "hbicg_solver_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.POINTER(Stats)]),
        "hbicg_solve": (C.c_int, [C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, C.c_int, C.POINTER(Params), C.c_void_p, C.c_void_p, C.POINTER(Stats)]),
        "hbicg_dropin_config": (None, [C.c_double, C.c_int, C.c_int]),
        "hbicg_true_residuals_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_void_p,
                                                   C.c_int, C.c_void_p, C.c_void_p]),
        "shifted_lopbicg_dynamic": (C.c_int, [C.POINTER(CSR_Matrix), C.POINTER(CSR_Matrix), C.POINTER(INFO_Matrix),
                                              _PD, _PD, _PD, C.c_int, C.c_int]),
        "shifted_lopbicg_static": (C.c_int, [C.POINTER(CSR_Matrix), C.POINTER(CSR_Matrix), C.POINTER(INFO_Matrix),
                                             _PD, _PD, _PD, C.c_int, C.c_int]),
        "shifted_lopbicg_normal": (C.c_int, [C.POINTER(CSR_Matrix), C.POINTER(CSR_Matrix), C.POINTER(INFO_Matrix),
                                             _PD, _PD, _PD, C.c_int, C.c_int]),
        "mult": (None, [C.POINTER(CSR_Matrix), _PD, _PD]),
        "mm_read_banner": (C.c_int, [C.c_void_p, C.c_void_p]),
        "mm_read_mtx_crd_size": (C.c_int, [C.c_void_p, _PI, _PI, _PI]),
        "csr_load_matrix": (C.c_int, [C.c_char_p, C.POINTER(CSR_Matrix)]),
        "MPI_csr_load_matrix_block": (None, [C.c_char_p, C.POINTER(CSR_Matrix), C.POINTER(CSR_Matrix),
                                             C.POINTER(INFO_Matrix)]),
        "csr_free_matrix": (None, [C.POINTER(CSR_Matrix)]),
        "coo2csr": (None, [C.POINTER(COO_Matrix), C.POINTER(CSR_Matrix)]),
        "csr_init_matrix": (None, [C.POINTER(CSR_Matrix)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int, what: str) -> None:
    if rc != 0:
        L = lib()
        raise HbicgError(f"{what}: {L.hbicg_status_string(rc).decode()} ({L.hbicg_last_message().decode()})")


def _ptr(a) -> int:
    """Address of a contiguous numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())


def params(tol=1e-12, max_iter=2000, switching=True, form="fused", shift_mode="auto", use_graph=True,
           graph_chunk=0, basis_mem_frac=0.0, true_residuals=False, basis_block=0, flush="auto",
           refine=True) -> Params:
    p = Params()
    lib().hbicg_params_default(C.byref(p))
    p.tol = float(tol)
    p.max_iter = int(max_iter)
    p.switching = 1 if switching else 0
    p.form = FORMS[form]
    p.shift_mode = SHIFT_MODES[shift_mode]
    # True: graphs of iteration chunks; "loop": one graph with a device-side
    # loop; "persistent": one persistent cooperative launch per solve
    p.use_graph = {"loop": 2, "persistent": 3}.get(use_graph, 1 if use_graph else 0) if isinstance(use_graph, str) \
        else (1 if use_graph else 0)
    p.graph_chunk = int(graph_chunk)
    if basis_mem_frac:
        p.basis_mem_frac = float(basis_mem_frac)
    p.true_residuals = 1 if true_residuals else 0
    p.basis_block = int(basis_block)
    p.flush_mode = FLUSH_MODES[flush]
    p.refine = 1 if refine else 0
    return p


# SpMV storage forms (hbicg_spmv_format)
_FORMATS = {0: "tile", 1: "sell", 2: "hyb", 3: "merge"}


@dataclass
class SolveResult:
    k: int
    x: object
    r: object
    status: int
    switches: list
    conv_k: np.ndarray
    active: np.ndarray
    final_seed: int
    shift_mode: str
    solve_ms: float
    flush_ms: float
    launches: int
    flushes: int
    bytes_algorithmic: float
    flush_bytes: float = 0.0
    refined: int = 0
    true_residual: np.ndarray | None = None
    extra: dict = field(default_factory=dict)

    @property
    def max_true_residual(self) -> float:
        return float(np.max(self.true_residual)) if self.true_residual is not None and len(self.true_residual) else 0.0


def _stats(m: int, max_iter: int):
    st = Stats()
    bufs = {
        "switch_k": np.zeros(max(m, 1), dtype=np.int32),
        "switch_seed": np.zeros(max(m, 1), dtype=np.int32),
        "conv_k": np.zeros(max(m, 1), dtype=np.int32),
        "active_per_iter": np.zeros(max_iter + 2, dtype=np.int32),
        "true_residual": np.zeros(max(m, 1)),
        "seed_alpha": np.zeros(max_iter + 2),
        "seed_beta": np.zeros(max_iter + 2),
        "seed_omega": np.zeros(max_iter + 2),
        "seed_rr": np.zeros(max_iter + 2),
    }
    st.switch_k = bufs["switch_k"].ctypes.data_as(_PI)
    st.switch_seed = bufs["switch_seed"].ctypes.data_as(_PI)
    st.conv_k = bufs["conv_k"].ctypes.data_as(_PI)
    st.active_per_iter = bufs["active_per_iter"].ctypes.data_as(_PI)
    st.true_residual = bufs["true_residual"].ctypes.data_as(_PD)
    for key in ("seed_alpha", "seed_beta", "seed_omega", "seed_rr"):
        setattr(st, key, bufs[key].ctypes.data_as(_PD))
    return st, bufs


def _result(st: Stats, bufs, m, x, r, want_res) -> SolveResult:
    nsw = min(st.n_switches, m)
    sw = [(int(bufs["switch_k"][i]), int(bufs["switch_seed"][i])) for i in range(nsw)]
    return SolveResult(k=st.k, x=x, r=r, status=st.status, switches=sw, conv_k=bufs["conv_k"][:m].copy(),
                       active=bufs["active_per_iter"][:st.k + 1].copy(), final_seed=st.final_seed,
                       shift_mode={1: "incremental", 2: "deferred"}.get(st.shift_mode, "?"), solve_ms=st.solve_ms,
                       flush_ms=st.flush_ms,
                       launches=st.launches, flushes=st.basis_flushes, bytes_algorithmic=st.bytes_algorithmic,
                       flush_bytes=st.flush_bytes, refined=st.refined_shifts,
                       true_residual=bufs["true_residual"][:m].copy() if want_res else None,
                       extra={"hist": {"alpha": bufs["seed_alpha"][:st.k].copy(), "beta": bufs["seed_beta"][:st.k].copy(),
                                       "omega": bufs["seed_omega"][:st.k].copy(), "rr": bufs["seed_rr"][:st.k].copy()}})


def _csr_arrays(a):
    return (np.ascontiguousarray(a.ptr, dtype=np.uint32), np.ascontiguousarray(a.col, dtype=np.uint32),
            np.ascontiguousarray(a.val, dtype=np.float64))


def solve(a, b, sigma, seed=0, *, tol=1e-12, max_iter=2000, switching=True, form="fused", shift_mode="auto",
          use_graph=True, true_residuals=False, graph_chunk=0, basis_mem_frac=0.0, basis_block=0,
          flush="auto", refine=True) -> SolveResult:
    """One-call solve with host (numpy) arrays through hbicg_solve."""
    L = lib()
    ptr, col, val = _csr_arrays(a)
    n, m = int(ptr.shape[0] - 1), len(sigma)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    x = np.zeros((m, n))
    r = np.zeros(n)
    p = params(tol, max_iter, switching, form, shift_mode, use_graph, graph_chunk, basis_mem_frac, true_residuals,
               basis_block, flush, refine)
    st, bufs = _stats(m, max_iter)
    rc = L.hbicg_solve(n, int(ptr[-1]), _ptr(ptr), _ptr(col), _ptr(val), _ptr(bb), _ptr(sig), m, int(seed),
                       C.byref(p), _ptr(x), _ptr(r), C.byref(st))
    if rc not in (0, 3, 4):
        _check(rc, "hbicg_solve")
    return _result(st, bufs, m, x, r, true_residuals)


def adjoint(a, b, sigma, w, c, seed: int = 0, same_context: bool = False, **kw) -> dict:
    """J = sum_j w_j c^T x_j for (A + sigma_j I) x_j = b and its gradients
    with respect to A's values (on its pattern), b and the shifts
    (hbicg_adjoint: one forward family, one transposed family, at once on two
    contexts; same_context: A^T made here on A's context, so the two families
    run one after the other).  numpy in/out."""
    ptr, col, val = _csr_arrays(a)
    n, m = int(ptr.shape[0] - 1), len(sigma)
    ctx = Context()
    A = Matrix(ctx, ptr, col, val)
    At = A.transpose() if same_context else None
    p = params(**kw)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    ww = np.ascontiguousarray(w, dtype=np.float64)
    cc = np.ascontiguousarray(c, dtype=np.float64)
    J = C.c_double()
    dval, db, ds, x = np.zeros(int(ptr[-1])), np.zeros(n), np.zeros(m), np.zeros((m, n))
    rc = lib().hbicg_adjoint(A.h, At.h if At is not None else None, _ptr(bb), _ptr(sig), m, int(seed), _ptr(ww),
                             _ptr(cc), C.byref(p), C.byref(J), _ptr(dval), _ptr(db), _ptr(ds), _ptr(x), None, None)
    if At is not None:
        At.close()
    A.close()
    ctx.close()
    if rc not in (0, 4):
        _check(rc, "hbicg_adjoint")
    return {"J": J.value, "dval": dval, "db": db, "dsigma": ds, "x": x, "status": rc}


def shifted_solve(ptr, col, val, b, sigma, seed: int = 0, **kw):
    """X = [x_j] with (A + sigma_j I) x_j = b as a differentiable torch op
    (val, b, sigma: float64 CUDA tensors; ptr, col: int32 CUDA tensors of A's
    pattern).  Backward: the transposed family (see torch_ops.py)."""
    from . import torch_ops

    return torch_ops.shifted_solve(ptr, col, val, b, sigma, seed, **kw)


@dataclass
class FamilyResult:
    status: int
    k: int
    x: np.ndarray
    switches: int
    final_seed: int
    spmv_format: str
    solve_ms: float
    wall_ms: float
    max_true_residual: float
    true_residual: np.ndarray | None
    message: str | None = None  # the first failing family (in order): what its failing call reported


def batch_solve(families, workers: int = 8, autotune: bool = False, autotune_cache: str | None = None,
                persistent: bool = True, persistent_ctas: int = 0, **kw) -> tuple[list, float]:
    """hbicg_batch_solve_opts over workloads.Family-like objects (a, b,
    sigma, seed): every family solved with the same parameters (kw as
    params()); persistent: the incremental-mode families share one persistent
    launch ("all": every family, both shift modes; False: none;
    persistent_ctas caps its CTAs, 0 = one wave).
    Returns ([FamilyResult], wall seconds)."""
    p = params(**kw)
    want_res = bool(kw.get("true_residuals", False))
    arr = (Family * max(len(families), 1))()
    keep = []
    for i, f in enumerate(families):
        ptr, col, val = _csr_arrays(f.a)
        b = np.ascontiguousarray(f.b, dtype=np.float64)
        sig = np.ascontiguousarray(f.sigma, dtype=np.float64)
        n, m = int(ptr.shape[0] - 1), len(sig)
        x = np.zeros((m, n))
        res = np.zeros(max(m, 1))
        keep.append((ptr, col, val, b, sig, x, res))
        fa = arr[i]
        fa.n, fa.nnz = n, int(ptr[-1])
        fa.ptr, fa.col, fa.val = ptr.ctypes.data_as(_PU), col.ctypes.data_as(_PU), val.ctypes.data_as(_PD)
        fa.b, fa.sigma = b.ctypes.data_as(_PD), sig.ctypes.data_as(_PD)
        fa.m, fa.seed, fa.autotune = m, int(f.seed), 1 if autotune else 0
        fa.x = x.ctypes.data_as(_PD)
        fa.true_residual = res.ctypes.data_as(_PD) if want_res else None
    wall = C.c_double()
    opts = BatchOpts()
    lib().hbicg_batch_opts_default(C.byref(opts))
    opts.workers = int(workers)
    opts.persistent = 2 if persistent == "all" else (1 if persistent else 0)
    opts.persistent_ctas = int(persistent_ctas)
    opts.autotune_cache = str(autotune_cache).encode() if autotune_cache else None
    rc = lib().hbicg_batch_solve_opts(arr, len(families), C.byref(p), C.byref(opts), C.byref(wall))
    msg = lib().hbicg_last_message().decode(errors="replace") if rc != 0 else None
    out = []
    for i in range(len(families)):
        fa = arr[i]
        out.append(FamilyResult(status=fa.status, k=fa.k, x=keep[i][5], switches=fa.n_switches,
                                final_seed=fa.final_seed, spmv_format=_FORMATS.get(fa.spmv_format, "tile"),
                                solve_ms=fa.solve_ms, wall_ms=fa.wall_ms, max_true_residual=fa.max_true_residual,
                                true_residual=keep[i][6][:len(keep[i][4])].copy() if want_res else None))
    if msg is not None:
        first = next((r for r in out if r.status != 0), None)
        if first is not None:
            first.message = msg
    return out, wall.value / 1e3


class Context:
    def __init__(self):
        self.h = C.c_void_p()
        _check(lib().hbicg_context_create(C.byref(self.h)), "hbicg_context_create")

    @property
    def stream(self) -> int:
        return int(lib().hbicg_context_stream(self.h) or 0)

    def close(self):
        if self.h:
            lib().hbicg_context_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Matrix:
    """Device CSR + SpMV schedule.  ptr/col/val: numpy (copied) or torch CUDA tensors (used in place)."""

    @classmethod
    def _wrap(cls, ctx: Context, h) -> "Matrix":
        self = cls.__new__(cls)
        self.ctx = ctx
        self._keep = ()
        self.h = h
        self.n = int(lib().hbicg_matrix_rows(h))
        self.nnz = int(lib().hbicg_matrix_nnz(h))
        return self

    @classmethod
    def from_coo(cls, ctx: Context, n: int, row, col, val) -> "Matrix":
        """CSR built on the GPU from triplets (numpy host arrays or torch CUDA
        tensors): row order, entries of a row in their given order."""
        where = HOST if isinstance(row, np.ndarray) else DEVICE
        if where == HOST:
            row = np.ascontiguousarray(row, dtype=np.uint32)
            col = np.ascontiguousarray(col, dtype=np.uint32)
            val = np.ascontiguousarray(val, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().hbicg_matrix_from_coo(ctx.h, int(n), int(row.shape[0]), _ptr(row), _ptr(col), _ptr(val), where,
                                           C.byref(h)), "hbicg_matrix_from_coo")
        return cls._wrap(ctx, h)

    @classmethod
    def load_mm(cls, ctx: Context, path: str, expand_symmetric: bool = False) -> "Matrix":
        """Matrix Market file -> device CSR (parallel parse, GPU COO -> CSR)."""
        h = C.c_void_p()
        _check(lib().hbicg_matrix_load_mm(ctx.h, str(path).encode(), int(bool(expand_symmetric)), C.byref(h)),
               "hbicg_matrix_load_mm")
        return cls._wrap(ctx, h)

    def transpose(self) -> "Matrix":
        """A^T on the same context, built on the GPU (stable by column)."""
        h = C.c_void_p()
        _check(lib().hbicg_matrix_transpose(self.h, C.byref(h)), "hbicg_matrix_transpose")
        return Matrix._wrap(self.ctx, h)

    def adjoint_gradients(self, X, Lam, w=None, want=("val", "b", "sigma")):
        """Gradients from solutions (torch CUDA tensors, [m, n] each): X with
        (A + sigma_j I) x_j = b, Lam with (A^T + sigma_j I) lam_j = g_j.
        Returns (dval [nnz], db [n], dsigma [m]) as CUDA tensors."""
        import torch

        m = int(X.shape[0])
        dev = X.device
        dval = torch.empty(self.nnz, dtype=torch.float64, device=dev) if "val" in want else None
        db = torch.empty(self.n, dtype=torch.float64, device=dev) if "b" in want else None
        ds = torch.empty(m, dtype=torch.float64, device=dev) if "sigma" in want else None
        _check(lib().hbicg_adjoint_gradients(self.h, m, _ptr(X), int(X.stride(0)), _ptr(Lam), int(Lam.stride(0)),
                                             _ptr(w) if w is not None else None,
                                             _ptr(dval) if dval is not None else None,
                                             _ptr(db) if db is not None else None,
                                             _ptr(ds) if ds is not None else None), "hbicg_adjoint_gradients")
        return dval, db, ds

    @property
    def format(self) -> str:
        return _FORMATS.get(lib().hbicg_matrix_format(self.h), "tile")

    def set_format(self, fmt: str) -> None:
        _check(lib().hbicg_matrix_set_format(self.h, {v: k for k, v in _FORMATS.items()}[fmt]), "hbicg_matrix_set_format")

    def autotune(self, cache: str | None = None) -> dict:
        """Time both SpMV forms (or read the cached choice) and keep the faster."""
        ch, t1, t2 = C.c_int(), C.c_double(), C.c_double()
        _check(lib().hbicg_matrix_autotune(self.h, str(cache).encode() if cache else None, C.byref(ch), C.byref(t1),
                                           C.byref(t2)), "hbicg_matrix_autotune")
        return {"format": _FORMATS.get(ch.value, "tile"), "tile_ms": t1.value, "sell_ms": t2.value}

    def csr(self):
        """(ptr, col, val) copied to numpy."""
        ptr = np.zeros(self.n + 1, dtype=np.uint32)
        col = np.zeros(self.nnz, dtype=np.uint32)
        val = np.zeros(self.nnz, dtype=np.float64)
        _check(lib().hbicg_matrix_get_csr(self.h, _ptr(ptr), _ptr(col), _ptr(val), HOST), "hbicg_matrix_get_csr")
        return ptr, col, val

    def __init__(self, ctx: Context, ptr, col, val):
        self.ctx = ctx
        self._keep = (ptr, col, val)
        where = HOST if isinstance(ptr, np.ndarray) else DEVICE
        if where == HOST:
            ptr = np.ascontiguousarray(ptr, dtype=np.uint32)
            col = np.ascontiguousarray(col, dtype=np.uint32)
            val = np.ascontiguousarray(val, dtype=np.float64)
            self._keep = (ptr, col, val)
        self.n = int(ptr.shape[0] - 1)
        self.nnz = int(col.shape[0])
        self.h = C.c_void_p()
        _check(lib().hbicg_matrix_create(ctx.h, self.n, self.nnz, _ptr(ptr), _ptr(col), _ptr(val), where,
                                         C.byref(self.h)), "hbicg_matrix_create")

    def spmv(self, x, y, sigma: float = 0.0):
        where = HOST if isinstance(x, np.ndarray) else DEVICE
        _check(lib().hbicg_matrix_spmv(self.h, _ptr(x), _ptr(y), float(sigma), where), "hbicg_matrix_spmv")
        return y

    def time_spmv(self, x, y, sigma: float = 0.0, iters: int = 20) -> float:
        """Mean milliseconds per SpMV launch (device tensors), CUDA events on the context stream."""
        if isinstance(x, np.ndarray) or isinstance(y, np.ndarray):
            raise TypeError("time_spmv takes device tensors; spmv takes host arrays")
        ms = C.c_double()
        _check(lib().hbicg_matrix_time_spmv(self.h, _ptr(x), _ptr(y), float(sigma), int(iters), C.byref(ms)),
               "hbicg_matrix_time_spmv")
        return ms.value

    def close(self):
        if self.h:
            lib().hbicg_matrix_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Reusable workspace for m-shift families on one matrix (graphs are captured once)."""

    def __init__(self, matrix: Matrix, m: int, **kw):
        self.matrix = matrix
        self.m = m
        self.max_iter = kw.get("max_iter", 2000)
        self.want_res = bool(kw.get("true_residuals", False))
        self.p = params(**kw)
        self.h = C.c_void_p()
        _check(lib().hbicg_solver_create(matrix.ctx.h, matrix.h, m, C.byref(self.p), C.byref(self.h)),
               "hbicg_solver_create")

    def run(self, b, sigma, seed=0, x=None, r=None) -> SolveResult:
        """b/sigma: numpy (host) or torch CUDA tensors (device); x [m, n] and r [n]
        are written in the same kind of memory as given (allocated on the host if None)."""
        in_where = HOST if isinstance(b, np.ndarray) else DEVICE
        if in_where == HOST:
            b = np.ascontiguousarray(b, dtype=np.float64)
            sigma = np.ascontiguousarray(sigma, dtype=np.float64)
        if x is None:
            x = np.zeros((self.m, self.matrix.n))
        out_where = HOST if isinstance(x, np.ndarray) else DEVICE
        st, bufs = _stats(self.m, self.max_iter)
        rc = lib().hbicg_solver_run(self.h, _ptr(b), _ptr(sigma), int(seed), in_where, _ptr(x),
                                    _ptr(r) if r is not None else None, out_where, C.byref(st))
        if rc not in (0, 3, 4):
            _check(rc, "hbicg_solver_run")
        return _result(st, bufs, self.m, x, r, self.want_res)

    def close(self):
        if self.h:
            lib().hbicg_solver_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------- reference entry points
def dropin_solve(variant: str, a, b, sigma, seed=0, tol=1e-12, max_iter=2000, switching=True):
    """Call shifted_lopbicg_<variant> exactly as the reference's drivers do
    (src/main.c:114-151): x zero, r_loc = b (overwritten), returns (k, x, r)."""
    L = lib()
    ptr, col, val = _csr_arrays(a)
    n, m = int(ptr.shape[0] - 1), len(sigma)
    diag = CSR_Matrix(val.ctypes.data_as(_PD), col.ctypes.data_as(_PU), ptr.ctypes.data_as(_PU), int(ptr[-1]), n, n)
    optr = np.zeros(n + 1, dtype=np.uint32)
    offd = CSR_Matrix(None, None, optr.ctypes.data_as(_PU), 0, n, n)
    recv = (C.c_int * 1)(n)
    displ = (C.c_int * 1)(0)
    info = INFO_Matrix(int(ptr[-1]), n, n, b"MCRG", C.cast(recv, _PI), C.cast(displ, _PI))
    x = np.zeros((m, n))
    r = np.ascontiguousarray(b, dtype=np.float64).copy()
    sig = np.ascontiguousarray(sigma, dtype=np.float64)
    L.hbicg_dropin_config(float(tol), int(max_iter), 1 if switching else 0)
    fn = getattr(L, f"shifted_lopbicg_{variant}")
    k = fn(C.byref(diag), C.byref(offd), C.byref(info), x.ctypes.data_as(_PD), r.ctypes.data_as(_PD),
           sig.ctypes.data_as(_PD), m, int(seed))
    L.hbicg_dropin_config(1e-12, 2000, 1)
    return k, x, r


def _check_noalloc_args(n: int, x, b, sigma, res) -> None:
    """Shape, dtype, layout and device rules of true_residuals_noalloc."""
    import torch

    named = {"x": x, "b": b, "sigma": sigma, "res": res}
    for name, t in named.items():
        if not isinstance(t, torch.Tensor):
            raise ValueError(f"{name} must be a torch tensor")
        if t.dtype != torch.float64:
            raise ValueError(f"{name} must be float64, got {t.dtype}")
    if sigma.dim() != 1:
        raise ValueError("sigma must be one-dimensional")
    m = int(sigma.shape[0])
    if x.dim() != 2 or int(x.shape[0]) != m:
        raise ValueError(f"x must have shape (m, >= n) with m = {m}, got {tuple(x.shape)}")
    if m and (int(x.shape[1]) < n or (int(x.shape[1]) > 1 and x.stride(1) != 1) or x.stride(0) < n):
        raise ValueError(f"x must hold m rows of at least n = {n} values with unit inner stride")
    for name, t, need in (("b", b, n), ("sigma", sigma, m), ("res", res, m)):
        if t.numel() < need:
            raise ValueError(f"{name} has {t.numel()} values, needs {need}")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    for name, t in named.items():
        if not t.is_cuda:
            raise ValueError(f"{name} must be on a CUDA device")


def true_residuals_noalloc(matrix: "Matrix", x, b, sigma, res, stream: int = 0) -> None:
    """hbicg_true_residuals_noalloc: res[j] = ||b - (A + sigma_j I) x_j|| / ||b||
    for device tensors x [m, ldx], b [n], sigma [m] and res [m], queued on
    `stream` without allocating device memory (at most 64 shifts).

    The arguments are checked here, before the call: float64 tensors on a CUDA
    device, x two-dimensional with m rows of at least n values and unit inner
    stride, b at least n values, sigma and res at least m values, each of b,
    sigma and res contiguous.  A tensor that breaks a rule raises ValueError
    instead of reaching the kernels, which would read or write past it."""
    _check_noalloc_args(matrix.n, x, b, sigma, res)
    m = int(sigma.shape[0])
    ldx = int(x.stride(0)) if m else matrix.n
    _check(lib().hbicg_true_residuals_noalloc(matrix.h, _ptr(x), ldx, _ptr(b), _ptr(sigma), m, _ptr(res),
                                              C.c_void_p(stream)), "hbicg_true_residuals_noalloc")


def release() -> None:
    """Return the device memory the library keeps between solves (its pool)."""
    lib().hbicg_release()


def dropin_raw(variant: str, ptr, col, val, x, r, sigma, seed=0, tol=1e-12, max_iter=2000, switching=True) -> int:
    """shifted_lopbicg_<variant> on caller-owned host buffers (numpy arrays or
    pinned torch CPU tensors, used in place): x [m, n] zero on entry, r = b on
    entry and the final seed residual on exit.  Returns the reference's k."""
    L = lib()
    n = int(ptr.shape[0] - 1)
    nz = int(col.shape[0])
    m = int(sigma.shape[0])
    diag = CSR_Matrix(C.cast(_ptr(val), _PD), C.cast(_ptr(col), _PU), C.cast(_ptr(ptr), _PU), nz, n, n)
    optr = np.zeros(n + 1, dtype=np.uint32)
    offd = CSR_Matrix(None, None, optr.ctypes.data_as(_PU), 0, n, n)
    recv = (C.c_int * 1)(n)
    displ = (C.c_int * 1)(0)
    info = INFO_Matrix(nz, n, n, b"MCRG", C.cast(recv, _PI), C.cast(displ, _PI))
    L.hbicg_dropin_config(float(tol), int(max_iter), 1 if switching else 0)
    try:
        fn = getattr(L, f"shifted_lopbicg_{variant}")
        return fn(C.byref(diag), C.byref(offd), C.byref(info), C.cast(_ptr(x), _PD), C.cast(_ptr(r), _PD),
                  C.cast(_ptr(sigma), _PD), m, int(seed))
    finally:
        L.hbicg_dropin_config(1e-12, 2000, 1)


def mult(a, x, y=None) -> np.ndarray:
    """The reference's mult (y += A x) through the C ABI, on the GPU."""
    L = lib()
    ptr, col, val = _csr_arrays(a)
    n = int(ptr.shape[0] - 1)
    A = CSR_Matrix(val.ctypes.data_as(_PD), col.ctypes.data_as(_PU), ptr.ctypes.data_as(_PU), int(ptr[-1]), n, n)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    yy = np.zeros(n) if y is None else np.ascontiguousarray(y, dtype=np.float64)
    L.mult(C.byref(A), xx.ctypes.data_as(_PD), yy.ctypes.data_as(_PD))
    return yy


def read_mm(path: str, expand_symmetric: bool = False, threads: int = 0) -> dict:
    """Parallel Matrix Market read (hbicg_mm_read) -> dict of numpy arrays
    row, col (0-based), val in file order, plus rows, cols, field, symmetry."""
    c = Coo()
    _check(lib().hbicg_mm_read(str(path).encode(), int(bool(expand_symmetric)), int(threads), C.byref(c)),
           "hbicg_mm_read")
    try:
        nnz = int(c.nnz)
        out = {"rows": int(c.rows), "cols": int(c.cols), "field": ["real", "integer", "pattern"][c.field],
               "symmetry": ["general", "symmetric", "skew-symmetric"][c.symmetry], "expanded": bool(c.expanded),
               "row": np.ctypeslib.as_array(c.row, shape=(nnz,)).copy() if nnz else np.zeros(0, np.uint32),
               "col": np.ctypeslib.as_array(c.col, shape=(nnz,)).copy() if nnz else np.zeros(0, np.uint32),
               "val": np.ctypeslib.as_array(c.val, shape=(nnz,)).copy() if nnz else np.zeros(0)}
    finally:
        lib().hbicg_coo_free(C.byref(c))
    return out


def load_matrix_market(path: str):
    """MPI_csr_load_matrix_block on one rank -> (Csr of the whole matrix, typecode)."""
    L = lib()
    d, o = CSR_Matrix(), CSR_Matrix()
    recv = (C.c_int * 1)(0)
    displ = (C.c_int * 1)(0)
    info = INFO_Matrix(0, 0, 0, b"    ", C.cast(recv, _PI), C.cast(displ, _PI))
    L.MPI_csr_load_matrix_block(str(path).encode(), C.byref(d), C.byref(o), C.byref(info))
    n, nz = d.rows, d.nz
    ptr = np.ctypeslib.as_array(d.ptr, shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(d.col, shape=(nz,)).copy() if nz else np.zeros(0, np.uint32)
    val = np.ctypeslib.as_array(d.val, shape=(nz,)).copy() if nz else np.zeros(0)
    code = bytes(info.code).decode()
    onz = o.nz
    L.csr_free_matrix(C.byref(d))
    L.csr_free_matrix(C.byref(o))
    return workloads.Csr(ptr, col, val), code, int(onz)
