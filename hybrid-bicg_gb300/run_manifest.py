#!/usr/bin/env python
"""Manifest-driven runner for batches of shifted families.

Replaces the reference's sweep drivers, which hard-code their matrices, shift
lists and seeds in C (src/main_seed_diff.c:113-155, src/main_repeat.c,
src/main.c:16-17,85): one JSON manifest lists the families; every (family,
seed) pair is one run; all runs go to hbicg_batch_solve, which solves them
concurrently on one GPU.  One JSON line per run is printed (name, seed,
status, iterations, switches, times, true residuals), and each run's
solutions can be saved as .npy.

Manifest:
{
  "params": {"tol": 1e-10, "max_iter": 10000, "switching": true,
             "shift_mode": "auto", "true_residuals": true},
  "workers": 8,
  "autotune_cache": "spmv_tune.txt",          (optional; enables the autotuner)
  "families": [
    {"name": "cd3d-32",
     "matrix": "A.mtx"                         (Matrix Market file, square)
            | {"generator": "stencil_cd3d", "args": [32]},
     "shifts": [0.0, 0.01, ...]
            | {"linspace": [0.0, 0.15, 16]} | {"geomspace": [1e-4, 1.0, 64]},
     "rhs": "unit" (1/sqrt(n), the reference's b) | "ones" | {"normal": 7}
          | "b.npy",
     "seeds": [0, 5, 15],                      (default [0])
     "out": "results/"}                        (optional: x as <name>_seed<s>.npy)
  ]
}

    python hybrid-bicg_gb300/run_manifest.py manifest.json [--workers N]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(_HERE.parent))


def _package():
    import __graft_entry__ as graft

    return graft.load_package()


class Run:
    """One (family, seed) solve: a, b, sigma, seed (the workloads.Family fields)."""

    def __init__(self, name, a, b, sigma, seed, out=None):
        self.name, self.a, self.b, self.sigma, self.seed, self.out = name, a, b, sigma, seed, out


def _matrix(pkg, spec, base: Path, cache: dict):
    key = json.dumps(spec, sort_keys=True)
    if key in cache:
        return cache[key]
    if isinstance(spec, str):
        c = pkg.read_mm(str(base / spec))
        if c["rows"] != c["cols"]:
            raise ValueError(f"{spec}: {c['rows']} x {c['cols']} is not square")
        n = c["rows"]
        order = np.argsort(c["row"], kind="stable")  # the reference's row order
        ptr = np.zeros(n + 1, dtype=np.int64)
        np.add.at(ptr, c["row"].astype(np.int64) + 1, 1)
        a = pkg.workloads.Csr(np.cumsum(ptr).astype(np.uint32), c["col"][order], c["val"][order])
    elif isinstance(spec, dict) and "generator" in spec:
        gen = spec["generator"]
        if gen not in ("stencil_cd3d", "stencil_cd2d", "irregular_powerlaw"):
            raise ValueError(f"unknown generator {gen!r}")
        a = getattr(pkg.workloads, gen)(*spec.get("args", []), **spec.get("kwargs", {}))
    else:
        raise ValueError(f"bad matrix spec {spec!r}")
    cache[key] = a
    return a


def _shifts(spec) -> np.ndarray:
    if isinstance(spec, list):
        return np.asarray(spec, dtype=np.float64)
    if isinstance(spec, dict) and "linspace" in spec:
        lo, hi, m = spec["linspace"]
        return np.linspace(lo, hi, int(m))
    if isinstance(spec, dict) and "geomspace" in spec:
        lo, hi, m = spec["geomspace"]
        return np.geomspace(lo, hi, int(m))
    raise ValueError(f"bad shifts spec {spec!r}")


def _rhs(spec, n: int, base: Path) -> np.ndarray:
    if spec in (None, "unit"):
        return np.full(n, 1.0 / np.sqrt(n))
    if spec == "ones":
        return np.ones(n)
    if isinstance(spec, dict) and "normal" in spec:
        return np.random.default_rng(int(spec["normal"])).standard_normal(n)
    if isinstance(spec, str):
        b = np.load(base / spec)
        if b.shape != (n,):
            raise ValueError(f"{spec}: shape {b.shape}, expected ({n},)")
        return np.asarray(b, dtype=np.float64)
    raise ValueError(f"bad rhs spec {spec!r}")


def expand(manifest: dict, base: Path, pkg=None) -> list[Run]:
    """The runs of a manifest, in manifest order (family, then seed)."""
    pkg = pkg or _package()
    cache: dict = {}
    runs = []
    for i, fam in enumerate(manifest.get("families", [])):
        name = fam.get("name", f"family{i}")
        a = _matrix(pkg, fam["matrix"], base, cache)
        sigma = _shifts(fam["shifts"])
        b = _rhs(fam.get("rhs"), a.n, base)
        for s in fam.get("seeds", [0]):
            if not 0 <= int(s) < len(sigma):
                raise ValueError(f"{name}: seed {s} outside [0, {len(sigma)})")
            runs.append(Run(name, a, b, sigma, int(s), fam.get("out")))
    return runs


def run(manifest: dict, base: Path, workers: int | None = None, stream=sys.stdout) -> list[dict]:
    pkg = _package()
    runs = expand(manifest, base, pkg)
    prm = dict(manifest.get("params", {}))
    cache = manifest.get("autotune_cache")
    results, wall = pkg.batch_solve(runs, workers=int(workers or manifest.get("workers", 8)),
                                    autotune=bool(cache), autotune_cache=str(base / cache) if cache else None, **prm)
    lines = []
    for r, res in zip(runs, results):
        line = {"name": r.name, "seed": r.seed, "n": r.a.n, "nnz": r.a.nnz, "m": len(r.sigma),
                "status": res.status, "k": res.k, "switches": res.switches, "final_seed": res.final_seed,
                "spmv_format": res.spmv_format, "solve_ms": res.solve_ms, "wall_ms": res.wall_ms}
        if res.true_residual is not None:
            line["max_true_residual"] = float(np.max(res.true_residual)) if len(res.true_residual) else 0.0
        if r.out:
            d = base / r.out
            os.makedirs(d, exist_ok=True)
            np.save(d / f"{r.name}_seed{r.seed}.npy", res.x)
        lines.append(line)
        print(json.dumps(line), file=stream, flush=True)
    print(json.dumps({"runs": len(runs), "wall_s": wall}), file=stream, flush=True)
    return lines


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("manifest")
    ap.add_argument("--workers", type=int, default=None)
    args = ap.parse_args(argv)
    path = Path(args.manifest).resolve()
    run(json.loads(path.read_text()), path.parent, args.workers)


if __name__ == "__main__":
    main()
