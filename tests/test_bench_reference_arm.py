"""The reference arm of bench.py on CPU: the reference's algorithm (the C
restatement under oracle/) timed on the host cores, one JSON line in the
bench contract, printed by rank 0 alone when launched with several ranks."""
import json
import socket
import subprocess
import sys

from conftest import ROOT

ARGS = ["--impl", "reference", "--workload", "c1", "--scale", "10", "--steps", "1", "--warmup", "1"]


def _json_lines(out: str):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check_line(d):
    assert d["impl"] == "reference" and d["unit"] == "s" and d["value"] > 0
    assert d["higher_is_better"] is False and d["dtype"] == "f64"
    assert d["steps"] == 1 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == "s"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_one_process():
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_line(lines[0])


def test_reference_arm_two_ranks_rank0_prints():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--gpus", "2", *ARGS]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_line(lines[0])
    assert lines[0]["n_gpus"] == 2
