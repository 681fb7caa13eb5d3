#!/usr/bin/env python
"""Benchmark of the shifted BiCGStab solve on one GB300 (one JSON line).

Workload (default): the 256^3 convection-diffusion family — n = 16,777,216,
nnz = 117,047,296, 64 shifts geometric in [1e-4, 1], b ~ N(0,1) normalised,
tol 1e-10 on every shift, seed 0, dynamic seed switching.  Synthetic and
seeded (the reference ships no matrices).

A step is one complete solve of the family.  `value` is the time per step (s)
with matrix, b and sigma already resident in HBM; `e2e` is the same solve
through the reference-facing C ABI (shifted_lopbicg_dynamic) from pinned host
buffers, the matrix and b copied in and all 64 solutions copied out inside the
timed region.  Every working set is far larger than the 129 MB L2, so no flush
is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank solves its own copy of the family (replicas only:
the solve does not shard across GPUs); the step time is the max over ranks.
`--impl reference` times the reference's CPU solver (its C restatement, built
in oracle/) on the host cores for a bounded sample and prints the same line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__ as graft  # noqa: E402

METRIC = "time-to-solution, all shifts @1e-10 true rel. residual; SpMV HBM GB/s vs peak"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def peaks_bf16():
    """Dense BF16 tensor peak (TFLOP/s): the measured burst figure, else the fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"])
    return 1900.0


# ------------------------------------------------------------- distributed
class Dist:
    """Replica bookkeeping: barrier and max/sum reductions over ranks."""

    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend or ("nccl" if _cuda() else "gloo"))
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, value: float, op: str) -> float:
        if not self.pg:
            return value
        import torch

        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([value], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def aggregate(dist: Dist, step_s: float, units: float):
    """Whole-job step time (max over ranks) and units processed by all ranks."""
    return dist.reduce(step_s, "max"), dist.reduce(units, "sum")


def _cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


# ------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(mhz)) if mhz else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(mhz)}


# ------------------------------------------------------------- workload
MATRIX_KIND = {
    "c1": "3-D 7-point convection-diffusion, ",
    "c2": "3-D 7-point convection-diffusion, ",
    "c3": "power-law rows (Zipf 2.0, mean 16, up to 4000; 70 % random and 30 % near-diagonal columns, "
          "diagonally dominant), ",
}


def workload(name: str, scale):
    pkg = graft.load_package()
    return pkg, pkg.workloads.family(name, scale)


def workload_config(args, f, world: int) -> dict:
    """The `config` object of a bench line: the workload alone, identical for
    both arms (how each arm computes it is reported outside `config`)."""
    m = len(f.sigma)
    return {"workload": f"{args.workload}: {f.a.n} rows, {f.a.nnz} nonzeros, {MATRIX_KIND.get(args.workload, '')}"
                        f"{m} shifts in [{f.sigma.min():g}, {f.sigma.max():g}], tol {f.tol:g}, seed {f.seed}",
            "mode": args.mode, "parallelism": f"replicas x{world}",
            "l2": "working set >> 129 MB L2 (no flush needed)"}


def spmv_bytes(n: int, nnz: int) -> float:
    """Compulsory HBM bytes of one y = (A + sigma I) x: values and column
    indices once (12 B per nonzero), row pointers once, x read once, y written
    once (x's neighbours come from L2)."""
    return 12.0 * nnz + 4.0 * (n + 1) + 16.0 * n


# DRAM bytes (read + write) that ncu measured for one tensor-core flush launch,
# per algorithmic byte (basis slots once, x_j read and written, Pmat_j read and
# written), on `bench.py --kernel flush --n 2097152` (64 shifts, 51 slots).
FLUSH_TRAFFIC_PER_ALGORITHMIC_BYTE = 5.097 / 5.151


def flush_roofline(bytes_per_launch: float, ms_per_launch: float, n: int, m: int, hbm: float, peak_kind: str):
    """Roofline of the basis flush (the solve's dominant kernel in deferred
    mode): its compulsory HBM bytes per launch (basis slots once, x_j and
    Pmat_j of the shifts it forms: those not converged by the previous flush)
    over its device time per launch (CUDA events around every flush of the
    timed solves, the small live-list, slot-maximum and coefficient-digit
    kernels included).  The tensor-core
    work behind it is reported beside: 45 digit-pair products over K = 64 per
    48-element tile and group of 64 shifts, M = 128."""
    achieved = bytes_per_launch / (ms_per_launch * 1e-3) / 1e9
    tiles = -(-n // 48) * -(-m // 64)
    tflop = tiles * 2.0 * 128 * 48 * 45 * 64 / 1e12
    ratio = FLUSH_TRAFFIC_PER_ALGORITHMIC_BYTE
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": bytes_per_launch * ratio if ratio else None,
            "kernel": "k_flush_tc (basis -> x_j, p_j on tcgen05 BF16 digit products)",
            "bytes_per_launch": bytes_per_launch, "ms_per_launch": ms_per_launch, "peak_kind": peak_kind,
            "tensor_tflops": tflop / (ms_per_launch * 1e-3), "tensor_peak_tflops": peaks_bf16()}


# ------------------------------------------------------------- CPU baseline
def load_profile(name: str, f):
    """Convergence profile of the reference's algorithm on a named workload
    (tests/golden/<name>_profile.json, made by tests/golden/make_golden.py
    --profile <name> from the oracle): iterations and the number of non-seed
    shifts each iteration updates."""
    p = ROOT / "tests" / "golden" / f"{name}_profile.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    if len(d["conv_k"]) != len(f.sigma):
        return None
    d["source"] = f"reference-algorithm profile {p.name}"
    return d


def load_digest(name: str):
    """Digest of the reference's own full solve of a named workload
    (tests/golden/<name>_digest.npz, made by tests/golden/make_golden.py
    --digest <name>): k, the switch sequence, and every shift's values at
    seeded rows, norm and true residual."""
    p = ROOT / "tests" / "golden" / f"{name}_digest.npz"
    if not p.exists():
        return None
    d = np.load(p, allow_pickle=False)
    return {k: d[k] for k in d.files}


def digest_compare(dig: dict, x, k: int, switches) -> dict:
    """Solutions against the reference's at the digest's rows (x: (m, n) host
    or device array): max over shifts of max |x_j - x_ref_j| / max |x_ref_j|
    at those rows, the relative error of ||x_j||, k and the switch sequence."""
    idx = dig["idx"]
    if hasattr(x, "index_select"):  # a torch tensor: gather on its device
        import torch

        xs = x.index_select(1, torch.as_tensor(idx, device=x.device)).cpu().numpy()
        nrm = torch.linalg.vector_norm(x, dim=1).cpu().numpy()
    else:
        xs = np.asarray(x)[:, idx]
        nrm = np.linalg.norm(x, axis=1)
    want = dig["x_at"]
    err = np.max(np.abs(xs - want), axis=1) / np.maximum(np.max(np.abs(want), axis=1), 1e-300)
    want_sw = [tuple(int(v) for v in row) for row in dig["switches"].reshape(-1, 2)]
    return {"max_rel_err_at_rows": float(np.max(err)), "rows": int(len(idx)),
            "max_rel_err_norm": float(np.max(np.abs(nrm - dig["norm"]) / dig["norm"])),
            "k": int(k), "k_reference": int(dig["k"]),
            "switches_match": [tuple(s) for s in switches] == want_sw}


def _cpu_baseline_child(name, scale, profile):
    return cpu_baseline(graft.load_package().workloads.family(name, scale), profile)


def cpu_baseline_fresh(name: str, scale, profile):
    """cpu_baseline in a spawned process: the GPU arm's process holds torch
    and its OpenMP thread pool, which the oracle's OpenMP team would compete
    with; a fresh interpreter times it as the reference arm does."""
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(1) as pool:
        return pool.apply(_cpu_baseline_child, (name, scale, profile))


def cpu_baseline(f, profile=None, threads: int | None = None):
    """The reference's algorithm (its C restatement, oracle/, with the
    reference's OpenMP layout) on the host cores, on a bounded sample:
    the seed system alone for 1 and 3 iterations and all shifts for 1 and 3
    iterations; the differences are steady per-iteration costs with set-up
    cancelled.  Time-to-solution = iterations x seed cost + shift updates x
    per-shift cost, with the iteration count and the per-iteration number of
    running shifts taken from the reference algorithm's convergence profile
    (committed, or — for workloads without one — the seed system solved to
    convergence here and the shifts replayed from its scalars)."""
    orc = graft.load_oracle()
    orc.build(ref=False)
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    one = f.sigma[f.seed:f.seed + 1]

    def timed(sigma, iters):
        t0 = time.perf_counter()
        orc.solve(f.a, f.b, sigma, seed=0 if len(sigma) == 1 else f.seed, tol=f.tol, max_iter=iters)
        return time.perf_counter() - t0

    t_seed = {s: timed(one, s) for s in (1, 3)}
    t_all = {s: timed(f.sigma, s) for s in (1, 3)}
    per_seed = max(t_seed[3] - t_seed[1], 0.0) / 2.0
    per_all = max(t_all[3] - t_all[1], 0.0) / 2.0
    per_shift = max(per_all - per_seed, 0.0) / max(len(f.sigma) - 1, 1)
    source = profile.get("source", "given profile") if profile else ""
    if profile is None:
        bb = float(f.b @ f.b)
        run = orc.solve(f.a, f.b, one, seed=0, tol=f.tol, max_iter=f.max_iter)
        conv, act = orc.shift_profile(run.hist, f.sigma, f.seed, f.tol, bb)
        profile = {"k": int(run.k), "shift_updates": int(act.sum())}
        source = "seed solved to convergence here"
    iters = int(profile["k"]) - 1
    updates = int(profile["shift_updates"])
    est = iters * per_seed + updates * per_shift + t_seed[1] - per_seed
    sample = (f"bounded sample: seed system alone for 1 and 3 iterations ({t_seed[1]:.2f} s, {t_seed[3]:.2f} s), "
              f"all {len(f.sigma)} shifts for 1 and 3 iterations ({t_all[1]:.2f} s, {t_all[3]:.2f} s); "
              f"estimate = {iters} iterations x {per_seed * 1e3:.1f} ms + {updates} shift updates x "
              f"{per_shift * 1e3:.2f} ms + set-up ({source})")
    return {"value": est, "unit": "s", "cores": cores, "kind": "port", "sample": sample,
            "iterations": iters + 1, "shift_updates": updates}


# ------------------------------------------------------------- our arm
def run_ours(args, dist: Dist):
    import torch

    torch.cuda.set_device(dist.local)
    pkg, f = workload(args.workload, args.scale)
    n, nnz, m = f.a.n, f.a.nnz, len(f.sigma)
    form = "plain" if args.mode == "static" else "fused"
    use_graph = args.mode != "normal"
    # the metric is the true residual: check it after every solve and correct
    # the shifts whose recursive residual converged above it (params.refine)
    kw = dict(tol=f.tol, max_iter=f.max_iter, form=form, shift_mode=args.shift_mode, use_graph=use_graph,
              flush=args.flush, basis_block=args.basis_block, refine=not args.no_refine)
    ctx = pkg.Context()
    ptr = torch.from_numpy(f.a.ptr.astype(np.int32)).cuda()
    col = torch.from_numpy(f.a.col.astype(np.int32)).cuda()
    val = torch.from_numpy(f.a.val).cuda()
    A = pkg.Matrix(ctx, ptr, col, val)
    solver = pkg.Solver(A, m, **kw)
    b = torch.from_numpy(f.b).cuda()
    sig = torch.from_numpy(f.sigma).cuda()
    x = torch.empty((m, n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream)
    for _ in range(args.warmup):
        res = solver.run(b, sig, seed=f.seed, x=x)
    torch.cuda.synchronize()
    dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    flush_ms = 0.0
    flush_bytes = 0.0
    flush_launches = 0
    with Clocks(dist.local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            res = solver.run(b, sig, seed=f.seed, x=x)
            launches += res.launches
            flush_ms += res.flush_ms
            flush_bytes += res.flush_bytes
            # mid-solve flushes plus the final one
            flush_launches += (res.flushes + 1) if res.shift_mode == "deferred" else 0
        ev1.record(stream)
        torch.cuda.synchronize()
    dist.barrier()
    step_s = ev0.elapsed_time(ev1) / 1e3 / args.steps
    step_max, units = aggregate(dist, step_s, 1.0)

    # verification solve (not timed): every shift's true residual, and the
    # solutions against the reference's own full solve where its digest exists
    ver = pkg.Solver(A, m, **{**kw, "true_residuals": True})
    vres = ver.run(b, sig, seed=f.seed, x=x)
    ver.close()
    dig = load_digest(args.workload) if args.scale is None else None
    parity = digest_compare(dig, x, vres.k, vres.switches) if dig is not None else None

    # the plain per-kernel GPU form on the same GPU (shifted_lopbicg_static's
    # form: one launch per step of the reference's iteration, the scalars on
    # the host), same matrix and settings: one untimed solve, one timed, then
    # every shift's true residual without allocating
    plain = None
    if form == "fused" and not args.no_plain:
        ps = pkg.Solver(A, m, **{**kw, "form": "plain", "use_graph": False})
        ps.run(b, sig, seed=f.seed, x=x)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        pres = ps.run(b, sig, seed=f.seed, x=x)
        p1.record(stream)
        torch.cuda.synchronize()
        ps.close()
        plain_s = p0.elapsed_time(p1) / 1e3
        tres = torch.empty(m, dtype=torch.float64, device="cuda")
        if m <= 64:
            pkg.true_residuals_noalloc(A, x, b, sig, tres, stream=ctx.stream)
            torch.cuda.synchronize()
        plain = {"value": plain_s, "unit": "s", "iterations": pres.k, "launches": pres.launches,
                 "refined_shifts": pres.refined,
                 "max_true_residual": float(tres.max().item()) if m <= 64 else None,
                 "fused_speedup": plain_s / step_max}

    # SpMV kernel alone (same kernel as the solve's two products), CUDA events
    xs = torch.randn(n, dtype=torch.float64, device="cuda")
    ys = torch.empty_like(xs)
    spmv_ms = A.time_spmv(xs, ys, float(f.sigma[0]), iters=20)
    hbm, peak_kind = peaks()
    sb = spmv_bytes(n, nnz)
    spmv = {"bound": "hbm", "achieved": sb / (spmv_ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
            "frac": sb / (spmv_ms * 1e-3) / 1e9 / hbm, "traffic": None, "kernel": "k_spmv",
            "bytes_per_launch": sb, "ms_per_launch": spmv_ms, "peak_kind": peak_kind}
    # the whole solve against HBM: the fused schedule's compulsory bytes (two
    # products and the seed's vectors per iteration, basis slots, the final
    # transpose), the flushes' algorithmic bytes, and the true-residual check
    # after the solve (one product per shift, with refine on); one timed step
    solve_bytes = res.bytes_algorithmic + res.flush_bytes + (0.0 if args.no_refine else m * sb)
    solve_gbs = solve_bytes / (step_max if step_max > 0 else float("inf")) / 1e9
    roofline_solve = {"bound": "hbm", "achieved": solve_gbs, "peak": hbm, "unit": "GB/s", "frac": solve_gbs / hbm,
                      "bytes_per_solve": solve_bytes, "s_per_solve": step_max, "peak_kind": peak_kind,
                      "model": "per iteration 2 products + seed vectors (deferred: 13 n-vectors + 2 basis slots; "
                               "incremental: 17 n-vectors + 4 per running shift); deferred: + the first slot, "
                               "+ x_j written once (8 n m), + 8n(L + 4 live) per flush; + one product per shift "
                               "for the true-residual check"}
    # the dominant kernel: the basis flush or the two SpMVs per iteration,
    # whichever takes more of the solve's device time
    roofline = spmv
    spmv_share_ms = 2.0 * max(res.k - 1, 0) * spmv_ms * args.steps
    if flush_launches and flush_ms > 0 and flush_ms >= spmv_share_ms:
        roofline = flush_roofline(flush_bytes / flush_launches, flush_ms / flush_launches, n, m, hbm, peak_kind)

    # e2e through the reference-facing C ABI with pinned host buffers; the
    # device-side objects above are closed first (their memory goes back to
    # the library's pool, which the calls below reuse), one untimed warm-up call
    e2e = None
    res_k, res_format = res.k, A.format
    solver.close()
    A.close()
    ctx.close()
    if not args.no_e2e:
        h_ptr = torch.from_numpy(f.a.ptr).pin_memory()
        h_col = torch.from_numpy(f.a.col).pin_memory()
        h_val = torch.from_numpy(f.a.val).pin_memory()
        h_b = torch.from_numpy(f.b).pin_memory()
        h_sig = torch.from_numpy(f.sigma).pin_memory()
        h_x = torch.empty((m, n), dtype=torch.float64).pin_memory()
        h_r = torch.empty(n, dtype=torch.float64).pin_memory()
        e2e_steps = 3  # the median of three calls: one slow call on a shared host does not set the figure
        dist.barrier()
        e2e_times = []
        for i in range(e2e_steps + 1):
            # the caller's inputs per the reference's contract (x zero, r = b on
            # entry); the timed region is the call: every host<->device copy,
            # the device set-up, the solve and the teardown
            h_x.zero_()
            h_r.copy_(h_b)
            t0 = time.perf_counter()
            k = pkg.dropin_raw("dynamic", h_ptr, h_col, h_val, h_x, h_r, h_sig, f.seed, f.tol, f.max_iter)
            if i:  # the first call is the warm-up
                e2e_times.append(time.perf_counter() - t0)
        e2e_s = float(np.median(e2e_times))
        e2e_max, _ = aggregate(dist, e2e_s, 1.0)
        e2e = {"value": e2e_max, "unit": "s", "h2d_bytes_per_step": int(h_ptr.nbytes + h_col.nbytes + h_val.nbytes
                                                                          + h_b.nbytes + h_sig.nbytes),
               "d2h_bytes_per_step": int(h_x.nbytes + h_r.nbytes), "api": "shifted_lopbicg_dynamic", "k": int(k),
               "calls_s": [round(t, 4) for t in e2e_times]}
        # where the end-to-end time goes: the same sequence as the drop-in call
        # (context, matrix from host arrays, solver, solve with every x_j
        # copied out, teardown) through the extended API, phase by phase, once
        ph = {}
        h_x.zero_()
        t0 = time.perf_counter()
        pctx = pkg.Context()
        pA = pkg.Matrix(pctx, h_ptr.numpy(), h_col.numpy(), h_val.numpy())
        t1 = time.perf_counter()
        ps_ = pkg.Solver(pA, m, tol=f.tol, max_iter=f.max_iter, refine=False)
        t2 = time.perf_counter()
        pres = ps_.run(h_b.numpy(), h_sig.numpy(), seed=f.seed, x=h_x.numpy(), r=h_r.numpy())
        t3 = time.perf_counter()
        ps_.close()
        pA.close()
        pctx.close()
        t4 = time.perf_counter()
        ph = {"context_and_matrix_upload_s": t1 - t0, "solver_setup_s": t2 - t1,
              "solve_and_copy_out_s": t3 - t2, "device_solve_s": pres.solve_ms / 1e3, "teardown_s": t4 - t3,
              "total_s": t4 - t0}
        e2e["breakdown"] = ph
        if plain is not None:
            # the same call through shifted_lopbicg_static (the plain form), once
            h_x.zero_()
            h_r.copy_(h_b)
            t0 = time.perf_counter()
            kp = pkg.dropin_raw("static", h_ptr, h_col, h_val, h_x, h_r, h_sig, f.seed, f.tol, f.max_iter)
            plain["e2e"] = {"value": time.perf_counter() - t0, "unit": "s", "api": "shifted_lopbicg_static",
                            "k": int(kp)}
            plain["fused_e2e_speedup"] = plain["e2e"]["value"] / e2e_max

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        prof = load_profile(args.workload, f) if args.scale is None else None
        if prof is None:
            # the GPU solve's own profile (same algorithm; within rounding of the reference's)
            prof = {"k": int(vres.k), "shift_updates": int(np.sum(vres.active)), "source": "the GPU solve's profile"}
        cpu = cpu_baseline_fresh(args.workload, args.scale, prof)

    line = {
        "metric": METRIC, "value": step_max, "unit": "s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_max * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator; the reference ships no matrices)",
        "config": workload_config(args, f, dist.world),
        "implementation": {"form": form, "graphs": use_graph, "shift_mode": res.shift_mode,
                           "refine": not args.no_refine, "spmv_format": res_format},
        "iterations": res.k, "switches": res.switches, "refined_shifts": res.refined,
        "max_true_residual": vres.max_true_residual,
        "all_converged": bool(np.all(vres.conv_k > 0)),
        "solve_breakdown_ms": {"flush": flush_ms / args.steps},
        "vs_reference_digest": parity, "plain": plain,
        "roofline": roofline, "roofline_spmv": spmv, "roofline_solve": roofline_solve, "e2e": e2e,
        "gpu_launches": launches, "cpu_baseline": cpu,
        "clocks": clk.summary(),
    }
    return line


def run_reference(args, dist: Dist):
    """The reference's CPU path on the host cores (rank 0 only), measured to
    convergence: the reference's algorithm and OpenMP layout (the oracle's C
    restatement, bit-identical to the reference's own sources where those
    compile) solves the whole family once, on all host threads.  The timed
    steps partition that one solve: the solver stamps the wall clock after
    every iteration, step i covers iterations [k_i, k_(i+1)) of K near-equal
    consecutive ranges, the first step also carries the set-up (allocation,
    the copies of b into every p_j) and the last the teardown.  `value` is the
    whole solve (the sum of the steps); the warm-up steps are untimed
    one-iteration solves of the same family.  Where a quick projection says
    the full solve would not end within `--ref-budget` seconds, the bounded
    sample and cost model of cpu_baseline stand in, labelled as an estimate."""
    if dist.rank != 0:
        return None
    _, f = workload(args.workload, args.scale)
    orc = graft.load_oracle()
    orc.build(ref=False)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    base = {"impl": "reference", "metric": METRIC, "unit": "s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator; the reference ships no matrices)",
            "config": workload_config(args, f, dist.world),
            "implementation": {"code": "reference algorithm, C restatement + OpenMP (oracle/)", "cores": cores}}
    for _ in range(max(1, args.warmup)):
        orc.solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=1)
    # projection: two iterations with every shift running, times the expected count
    t0 = time.perf_counter()
    orc.solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=2)
    per_iter = (time.perf_counter() - t0) / 2.0
    prof = load_profile(args.workload, f) if args.scale is None else None
    k_expect = int(prof["k"]) if prof else f.max_iter
    projected = per_iter * k_expect
    if projected > args.ref_budget:
        info = cpu_baseline(f, prof)
        v = info["value"]
        return {**base, "value": v, "ms_per_step": v * 1e3, "measured": False,
                "projection_s": projected,
                "cpu_baseline": {**info, "kind": "port", "sample": "estimate (full solve projected beyond "
                                 f"{args.ref_budget:.0f} s): " + info["sample"]},
                "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    t0 = time.perf_counter()
    res = orc.solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=f.max_iter)
    total = time.perf_counter() - t0
    stamps = np.asarray(res.hist["t"], dtype=np.float64)  # [0]: iterations start, [k]: end of iteration k
    kk = len(stamps) - 1  # iterations done
    cuts = np.linspace(0, kk, args.steps + 1).round().astype(int)
    steps = [float(stamps[b] - stamps[a]) for a, b in zip(cuts[:-1], cuts[1:])]
    steps[0] += total - float(stamps[-1] - stamps[0])  # set-up and teardown outside the stamps
    tr = orc.true_residuals(f.a, res.x, f.b, f.sigma)
    sample = (f"one complete solve ({res.k - 1} iterations, all {len(f.sigma)} shifts, {cores} threads); "
              f"the {args.steps} timed steps are consecutive iteration ranges of it")
    line = {**base, "value": total, "ms_per_step": total / args.steps * 1e3, "measured": True,
            "step_s": [round(t, 3) for t in steps], "timed_region_s": total, "iterations": int(res.k),
            "switches": res.switches, "max_true_residual": float(np.max(tr)), "projection_s": projected,
            "cpu_baseline": {"value": total, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": total, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    dig = load_digest(args.workload) if args.scale is None else None
    if dig is not None:
        line["vs_reference_digest"] = digest_compare(dig, res.x, res.k, res.switches)
    return line


def run_batch_c4(args, dist: Dist):
    """Config 4: 256 uneven families (2-D 5-point / 3-D 7-point, n log-uniform
    in [1e4, 5e5], 8..64 shifts each) through hbicg_batch_solve: a step is the
    whole batch, from host arrays (matrices, b, sigma in; every x_j out), so
    the copies are inside the timed region and `value` is also the end-to-end
    figure.  The families that take the incremental shift mode share one
    persistent launch unless --no-persistent; the line also reports the same
    batch without it and the sequential per-family loop (one worker, one
    family on the GPU at a time).  CPU baseline: the reference's algorithm
    (oracle/) solved to convergence on a bounded sample of the cheapest
    families, costed per (nnz + 6 m n) x iterations and scaled to all 256 with
    the GPU's counts."""
    pkg = graft.load_package()
    fams = pkg.workloads.batched_families(256)
    kw = dict(tol=1e-10, max_iter=10000, shift_mode=args.shift_mode, flush=args.flush, true_residuals=True,
              refine=not args.no_refine, basis_block=args.basis_block,
              persistent=False if args.no_persistent else ("all" if args.persistent_all else True),
              persistent_ctas=args.persistent_ctas)
    for _ in range(max(1, args.warmup)):
        pkg.batch_solve(fams, workers=args.workers, **kw)
    walls, res = [], None
    with Clocks(dist.local) as clk:
        for _ in range(args.steps):
            res, wall = pkg.batch_solve(fams, workers=args.workers, **kw)
            walls.append(wall)
    value = float(np.median(walls))
    status_bad = sum(r.status != 0 for r in res)
    over = [i for i, r in enumerate(res) if r.max_true_residual > 1e-10 * 1.01]
    iters = int(sum(r.k for r in res))
    work = lambda f, k: (f.a.nnz + 6.0 * len(f.sigma) * f.a.n) * max(k - 1, 1)
    # the families of the shared persistent launch (incremental shift mode)
    in_group = lambda f: (not args.no_persistent and (args.persistent_all or (args.shift_mode == "auto"
                                                                              and f.a.n * len(f.sigma) < (1 << 21))))
    line = {"metric": "C4: time to solve 256 uneven shifted families (host arrays in/out), tol 1e-10",
            "value": value, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "c4: 256 families, n log-uniform in [1e4, 5e5] (2-D 5-point / 3-D 7-point "
                                   "convection-diffusion), 8..64 shifts uniform in [1e-3, 1], b ~ N(0,1)",
                       "workers": args.workers, "shift_mode": args.shift_mode, "refine": not args.no_refine,
                       "persistent": "none" if args.no_persistent else ("all" if args.persistent_all else "incremental"),
                       "persistent_ctas": args.persistent_ctas,
                       "l2": "every family's working set is re-read from HBM"},
            "persistent_families": sum(1 for f in fams if in_group(f)),
            "families_per_s": 256 / value, "total_iterations": iters, "status_failures": status_bad,
            "failed_families": [[i, int(r.status), int(r.k)] + ([r.message] if r.message else [])
                                for i, r in enumerate(res) if r.status != 0],
            "families_over_tol": over, "max_true_residual": max(r.max_true_residual for r in res),
            # device time of the worker-solved families, plus the shared launch once
            "sum_device_solve_s": (sum(r.solve_ms for f, r in zip(fams, res) if not in_group(f))
                                   + max([r.solve_ms for f, r in zip(fams, res) if in_group(f)] or [0.0])) / 1e3,
            "persistent_launch_s": max([r.solve_ms for f, r in zip(fams, res) if in_group(f)] or [0.0]) / 1e3,
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": int(sum(12 * f.a.nnz + 4 * (f.a.n + 1) + 8 * f.a.n
                                                                             + 8 * len(f.sigma) for f in fams)),
                    "d2h_bytes_per_step": int(sum(8 * len(f.sigma) * f.a.n for f in fams))},
            "clocks": clk.summary(), "cpu_baseline": None}
    # the same batch with every family on the workers (no shared launch), once
    if not args.no_persistent:
        w_res, w_wall = pkg.batch_solve(fams, workers=args.workers, **{**kw, "persistent": False})
        line["workers_only"] = {"value": w_wall, "unit": "s", "families_per_s": 256 / w_wall,
                                "status_failures": sum(r.status != 0 for r in w_res),
                                "persistent_speedup": w_wall / value}
    # the same families one after another through the same API on the same
    # GPU (one worker, no shared launch: one family on the device at a time), once
    seq_res, seq_wall = pkg.batch_solve(fams, workers=1, **{**kw, "persistent": False})
    line["sequential"] = {"value": seq_wall, "unit": "s", "families_per_s": 256 / seq_wall,
                          "status_failures": sum(r.status != 0 for r in seq_res),
                          "batched_speedup": seq_wall / value}
    if not args.no_cpu_baseline:
        orc = graft.load_oracle()
        orc.build(ref=False)
        cost = sorted(range(256), key=lambda i: work(fams[i], res[i].k))
        sample, t_cpu, units = [], 0.0, 0.0
        for i in cost:
            f = fams[i]
            t0 = time.perf_counter()
            r = orc.solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=f.max_iter)
            t_cpu += time.perf_counter() - t0
            units += work(f, r.k)
            sample.append(i)
            if t_cpu > 20.0 or len(sample) >= 24:
                break
        total_units = sum(work(f, r.k) for f, r in zip(fams, res))
        line["cpu_baseline"] = {"value": t_cpu / units * total_units, "unit": "s",
                                "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                                "kind": "port", "sample": f"the {len(sample)} cheapest families solved to convergence "
                                f"({t_cpu:.1f} s), scaled by (nnz + 6 m n) x iterations to all 256"}
    return line


def run_adjoint_c5(args, dist: Dist):
    """Config 5: J = sum_k w_k c^T x(sigma_k) on the 128^3 convection-diffusion
    matrix with 32 shifts, and its gradients with respect to A's values, b and
    the shifts (hbicg_adjoint: forward family, GPU transpose, transposed family
    on A^T with right-hand side c, gradient kernels).  A step is one call from
    host arrays (matrix, b, sigma, w, c in; J, the three gradients and all x_j
    out).  CPU baseline: the reference's algorithm for the forward family on a
    bounded sample (its cost model), counted twice (the transposed family has
    the same size and iteration count to within a few)."""
    pkg, f = workload("c5", args.scale)
    w, c = f.extra["w"], f.extra["c"]
    kw = dict(seed=f.seed, tol=f.tol, max_iter=f.max_iter)
    for _ in range(args.warmup):
        out = pkg.adjoint(f.a, f.b, f.sigma, w, c, **kw)
    times = []
    with Clocks(dist.local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = pkg.adjoint(f.a, f.b, f.sigma, w, c, **kw)
            times.append(time.perf_counter() - t0)
    value = float(np.median(times))
    n, m, nnz = f.a.n, len(f.sigma), f.a.nnz
    line = {"metric": "C5: J = sum_k w_k c^T x(sigma_k) and dJ/dval, dJ/db, dJ/dsigma (host arrays in/out)",
            "value": value, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": f"c5: {n} rows, {nnz} nonzeros, 3-D 7-point convection-diffusion, {m} shifts "
                                   f"uniform in [1e-3, 1], w ~ U(0,1), b, c ~ N(0,1), tol {f.tol:g}"},
            "status": out["status"], "J": out["J"],
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": int(12 * nnz + 4 * (n + 1) + 16 * n + 16 * m),
                    "d2h_bytes_per_step": int(8 * (nnz + n + m + m * n))},
            "clocks": clk.summary(), "cpu_baseline": None}
    # the forward family alone through the same kind of call (host arrays in,
    # every x_j out), for the cost of the gradients relative to the solve
    for _ in range(max(1, args.warmup)):
        pkg.solve(f.a, f.b, f.sigma, **kw)
    ftimes = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fwd = pkg.solve(f.a, f.b, f.sigma, **kw)
        ftimes.append(time.perf_counter() - t0)
    line["forward"] = {"value": float(np.median(ftimes)), "unit": "s", "iterations": int(fwd.k),
                       "api": "hbicg_solve (host arrays in, x out)"}
    line["adjoint_over_forward"] = value / line["forward"]["value"]
    if not args.no_cpu_baseline:
        fwd = pkg.solve(f.a, f.b, f.sigma, seed=f.seed, tol=f.tol, max_iter=f.max_iter)
        prof = {"k": int(fwd.k), "shift_updates": int(np.sum(fwd.active)), "source": "the GPU forward solve's profile"}
        cb = cpu_baseline_fresh("c5", args.scale, prof)
        cb["value"] *= 2.0
        cb["sample"] = "2 x (forward family) " + cb["sample"]
        line["cpu_baseline"] = cb
    return line


def run_flush_kernel(args):
    """The basis flush alone (hbk_flush_tc_run: slot maxima, coefficient
    digits, the tensor-core kernel) on random FP64 data of a solve's shape:
    n elements, 64 shifts, 51 basis slots, p kept, x_j and p_j panel-major
    as in a solve.  CUDA events around `--steps` calls after `--warmup`;
    algorithmic bytes 8 n (L + 4 m)."""
    import ctypes as C

    import torch

    pkg = graft.load_package()
    lib = pkg.lib()
    fn = lib.hbk_flush_tc_run
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_uint, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hbk_flush_tc_workspace_bytes.restype = C.c_size_t
    lib.hbk_flush_tc_workspace_bytes.argtypes = [C.c_int]
    n, m, L, cap = args.n, 64, 51, 72
    ld = (n + 31) // 32 * 32
    g = torch.Generator(device="cuda").manual_seed(0)
    V = torch.randn(L, ld, dtype=torch.float64, device="cuda", generator=g)
    panel_elems = -(-n // 48) * 48 * m  # panel-major x_j and p_j
    X = torch.randn(panel_elems, dtype=torch.float64, device="cuda", generator=g)
    P = torch.randn(panel_elems, dtype=torch.float64, device="cuda", generator=g)
    Xc = torch.randn(m, cap, dtype=torch.float64, device="cuda", generator=g)
    Pc = torch.randn(m, cap, dtype=torch.float64, device="cuda", generator=g)
    own = torch.randn(m, 2, dtype=torch.float64, device="cuda", generator=g)
    ws = torch.zeros(int(lib.hbk_flush_tc_workspace_bytes(m)) // 8 + 1, dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream

    def call():
        rc = fn(V.data_ptr(), ld, n, L, Xc.data_ptr(), Pc.data_ptr(), cap, own.data_ptr(), m, X.data_ptr(),
                P.data_ptr(), 1, ws.data_ptr(), err.data_ptr(), st)
        if rc:
            raise RuntimeError(f"hbk_flush_tc_run returned {rc}")

    for _ in range(args.warmup):
        call()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        call()
    e1.record()
    torch.cuda.synchronize()
    if int(err.item()):
        raise RuntimeError("tensor-core flush reported a wait timeout")
    ms = e0.elapsed_time(e1) / args.steps
    byt = 8.0 * n * (L + 4 * m)
    hbm, kind = peaks()
    # the FP64 product it stands in for: 2 m rows (x and p) x L slots x n, 2 flops each
    fp64_tflops = 2.0 * (2 * m) * L * n / (ms * 1e-3) / 1e12
    return {"kernel": "k_flush_tc", "n": n, "shifts": m, "slots": L, "ms_per_launch": ms, "bytes_per_launch": byt,
            "achieved_gbs": byt / (ms * 1e-3) / 1e9, "frac": byt / (ms * 1e-3) / 1e9 / hbm, "peak_kind": kind,
            "fp64_equivalent_tflops": fp64_tflops, "fp64_peak_tflops_measured_probe": 1.012}


def run_spmv_kernel(args):
    """y = (A + sigma I) x alone for a workload's matrix in each SpMV form the
    matrix has (tile always; SELL-32 where every row fits; HYB), device
    buffers, CUDA events over `--steps` launches after `--warmup`; algorithmic
    bytes 12 nnz + 4 (n + 1) + 16 n.  The default form comes first."""
    import torch

    pkg, f = workload(args.workload, args.scale)
    n, nnz = f.a.n, f.a.nnz
    ctx = pkg.Context()
    A = pkg.Matrix(ctx, torch.from_numpy(f.a.ptr.astype(np.int32)).cuda(),
                   torch.from_numpy(f.a.col.astype(np.int32)).cuda(), torch.from_numpy(f.a.val).cuda())
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(0))
    y = torch.empty_like(x)
    hbm, kind = peaks()
    byt = spmv_bytes(n, nnz)
    default = A.format
    out = {"kernel": "k_spmv", "workload": args.workload, "n": n, "nnz": nnz, "default_format": default,
           "bytes_per_launch": byt, "peak_kind": kind, "forms": {}}
    for fmt in [default] + [g for g in ("tile", "sell", "hyb", "merge") if g != default]:
        try:
            A.set_format(fmt)
        except RuntimeError:
            continue  # no such form for this matrix (SELL-32 with rows over 64 entries)
        ms = A.time_spmv(x, y, 0.1, iters=max(args.steps, 1))
        out["forms"][fmt] = {"ms_per_launch": ms, "achieved_gbs": byt / (ms * 1e-3) / 1e9,
                             "frac": byt / (ms * 1e-3) / 1e9 / hbm}
    A.set_format(default)
    A.close()
    if args.row_classes:
        # the same matrix with the rows of one length class emptied, default form
        ptr = f.a.ptr.astype(np.int64)
        lens = np.diff(ptr)
        rowlen = np.repeat(lens, lens)
        out["row_classes"] = {}
        for name, keep in (("rows_le_32", rowlen <= 32), ("rows_gt_32", rowlen > 32)):
            nl = np.bincount(np.repeat(np.arange(n), lens)[keep], minlength=n)
            p = np.zeros(n + 1, dtype=np.int64)
            np.cumsum(nl, out=p[1:])
            B = pkg.Matrix(ctx, p.astype(np.uint32), f.a.col[keep], f.a.val[keep])
            ms = min(B.time_spmv(x, y, 0.1, iters=max(args.steps, 1)) for _ in range(3))
            out["row_classes"][name] = {"nnz": int(keep.sum()), "format": B.format, "ms_per_launch": ms}
            B.close()
    ctx.close()
    return out


def run_coo2csr_kernel(args):
    """COO -> CSR of a workload's matrix (its triplets in a random order) on
    the GPU (hbk_coo_to_csr: stable radix sort by row, row pointers, gather;
    device buffers, CUDA events) beside the reference's host algorithm (a
    stable counting sort by row, then the row cut: coo2csr, one core)."""
    import ctypes as C

    import torch

    pkg, f = workload(args.workload, args.scale)
    a = f.a
    n, nnz = a.n, a.nnz
    rng = np.random.default_rng(0)
    perm = rng.permutation(nnz)
    row = np.repeat(np.arange(n, dtype=np.uint32), np.diff(a.ptr.astype(np.int64)))[perm]
    col = a.col.astype(np.uint32)[perm]
    val = a.val[perm]
    lib = pkg.lib()
    lib.hbk_coo_to_csr_tmp_bytes.restype = C.c_size_t
    lib.hbk_coo_to_csr_tmp_bytes.argtypes = [C.c_uint]
    fn = lib.hbk_coo_to_csr
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint, C.c_uint] + [C.c_void_p] * 8 + [C.c_void_p]
    d_row = torch.from_numpy(row.astype(np.int32)).cuda()
    d_col = torch.from_numpy(col.astype(np.int32)).cuda()
    d_val = torch.from_numpy(val).cuda()
    ptr = torch.empty(n + 1, dtype=torch.int32, device="cuda")
    col_o = torch.empty(nnz, dtype=torch.int32, device="cuda")
    val_o = torch.empty(nnz, dtype=torch.float64, device="cuda")
    tmp = torch.empty(int(lib.hbk_coo_to_csr_tmp_bytes(nnz)), dtype=torch.uint8, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream

    def call():
        rc = fn(n, nnz, d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), ptr.data_ptr(), col_o.data_ptr(),
                val_o.data_ptr(), tmp.data_ptr(), err.data_ptr(), st)
        if rc:
            raise RuntimeError(f"hbk_coo_to_csr returned {rc}")

    for _ in range(args.warmup):
        call()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ok = int(err.item()) == 0 and np.array_equal(ptr.cpu().numpy().astype(np.uint32), a.ptr.astype(np.uint32))
    # the reference's host algorithm on the same triplets
    coo = pkg.COO_Matrix()
    coo.val = val.ctypes.data_as(C.POINTER(C.c_double))
    coo.row = row.ctypes.data_as(C.POINTER(C.c_uint))
    coo.col = col.ctypes.data_as(C.POINTER(C.c_uint))
    coo.nz, coo.rows, coo.cols = nnz, n, n
    out = pkg.CSR_Matrix()
    t0 = time.perf_counter()
    lib.coo2csr(C.byref(coo), C.byref(out))
    host_s = time.perf_counter() - t0
    same = (np.array_equal(np.ctypeslib.as_array(out.ptr, shape=(n + 1,)), ptr.cpu().numpy().astype(np.uint32))
            and np.array_equal(np.ctypeslib.as_array(out.col, shape=(nnz,)), col_o.cpu().numpy().astype(np.uint32))
            and np.array_equal(np.ctypeslib.as_array(out.val, shape=(nnz,)), val_o.cpu().numpy()))
    lib.csr_free_matrix(C.byref(out))
    byt = 28.0 * nnz + 4.0 * (n + 1)  # triplets read once, col/val written once, ptr written
    hbm, kind = peaks()
    return {"kernel": "hbk_coo_to_csr", "workload": args.workload, "n": n, "nnz": nnz, "ms": ms,
            "entries_per_s": nnz / (ms * 1e-3), "algorithmic_gbs": byt / (ms * 1e-3) / 1e9,
            "frac": byt / (ms * 1e-3) / 1e9 / hbm, "peak_kind": kind, "error_flag": int(err.item()),
            "host_reference_algorithm_s": host_s, "identical_to_host": bool(same and ok)}


def run_mmread(args):
    """Matrix Market read of a workload's matrix: the parallel reader on all
    host cores beside the same reader on one core (the reference reads with one
    fscanf per entry on one core)."""
    import tempfile

    pkg, f = workload(args.workload, args.scale)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "a.mtx")
        t0 = time.perf_counter()
        pkg.workloads.write_matrix_market(path, f.a)
        write_s = time.perf_counter() - t0
        size = os.path.getsize(path)
        times = {}
        for th in (1, 0):
            best = None
            for _ in range(max(1, args.steps)):
                t0 = time.perf_counter()
                c = pkg.read_mm(path, threads=th)
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            times["all_cores" if th == 0 else "one_core"] = best
        same = len(c["val"]) == f.a.nnz
    return {"kernel": "hbicg_mm_read", "workload": args.workload, "n": f.a.n, "nnz": f.a.nnz, "file_bytes": size,
            "s_all_cores": times["all_cores"], "s_one_core": times["one_core"], "cores": os.cpu_count(),
            "speedup": times["one_core"] / times["all_cores"], "MB_per_s": size / times["all_cores"] / 1e6,
            "write_s": write_s, "entries_ok": bool(same)}


def run_group_kernel(args):
    """The shared persistent launch alone on a small case of config 4: the
    first `--families` (default 64) families of the 256-family batch that take
    the incremental shift mode, solved by hbicg_batch_solve_opts with the
    shared launch; `--warmup` untimed and `--steps` timed calls.  Reports the
    launch's device time (CUDA events around it) and the whole call's."""
    pkg = graft.load_package()
    fams = [f for f in pkg.workloads.batched_families(256) if f.a.n * len(f.sigma) < (1 << 21)][:args.families]
    kw = dict(tol=1e-10, max_iter=10000, true_residuals=True, persistent=True, persistent_ctas=args.persistent_ctas)
    for _ in range(args.warmup):
        pkg.batch_solve(fams, workers=args.workers, **kw)
    launch, wall, res = [], [], None
    for _ in range(max(1, args.steps)):
        res, w = pkg.batch_solve(fams, workers=args.workers, **kw)
        launch.append(res[0].solve_ms)
        wall.append(w)
    return {"kernel": "k_group (shared persistent launch)", "families": len(fams),
            "rows": int(sum(f.a.n for f in fams)), "shifts": int(sum(len(f.sigma) for f in fams)),
            "launch_ms": float(np.median(launch)), "call_s": float(np.median(wall)),
            "iterations_max": int(max(r.k for r in res)), "status_failures": sum(r.status != 0 for r in res),
            "max_true_residual": max(r.max_true_residual for r in res)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--scale", type=int, default=None, help="grid side override (smaller case of the same shape)")
    ap.add_argument("--mode", default="dynamic", choices=["dynamic", "static", "normal"])
    ap.add_argument("--shift-mode", default="auto", choices=["auto", "incremental", "deferred"])
    ap.add_argument("--flush", default="auto", choices=["auto", "fp64", "tensor"])
    ap.add_argument("--basis-block", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain per-kernel form beside the fused")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-refine", action="store_true", help="keep the reference's x (no true-residual correction)")
    ap.add_argument("--row-classes", action="store_true",
                    help="--kernel spmv: also time the matrix with its rows of <= 32 / > 32 entries emptied")
    ap.add_argument("--kernel", default=None, choices=["flush", "spmv", "coo2csr", "mmread", "group"],
                    help="time one kernel alone on random data instead of the solve")
    ap.add_argument("--n", type=int, default=2097152, help="elements for --kernel")
    ap.add_argument("--families", type=int, default=64, help="families for --kernel group")
    ap.add_argument("--workers", type=int, default=8, help="host workers for --workload c4")
    ap.add_argument("--no-persistent", action="store_true",
                    help="--workload c4: every family on the workers (no shared persistent launch)")
    ap.add_argument("--persistent-all", action="store_true",
                    help="--workload c4: every family in the shared persistent launch (both shift modes)")
    ap.add_argument("--persistent-ctas", type=int, default=0, help="CTAs of c4's persistent launch (0: one wave)")
    ap.add_argument("--ref-budget", type=float, default=1500.0,
                    help="--impl reference: longest projected full CPU solve (s) to measure; beyond it, estimate")
    args = ap.parse_args(argv)
    if args.kernel:
        run = {"flush": run_flush_kernel, "spmv": run_spmv_kernel, "coo2csr": run_coo2csr_kernel,
               "mmread": run_mmread, "group": run_group_kernel}[args.kernel]
        print(json.dumps(run(args)), flush=True)
        return
    if args.impl == "ours" and args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.workload == "c4" and args.impl == "ours":
            line = run_batch_c4(args, dist)
        elif args.workload == "c5" and args.impl == "ours":
            line = run_adjoint_c5(args, dist)
        else:
            line = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if line is not None and dist.rank == 0:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
