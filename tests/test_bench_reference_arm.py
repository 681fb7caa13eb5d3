"""bench.py's host side on CPU: the reference arm (the reference's algorithm,
the C restatement under oracle/, timed on the host cores) prints one JSON line
in the bench contract, from rank 0 alone when launched with several ranks; the
clocks object is read from nvidia-smi's sample lines."""
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
    # one complete solve measured, its steps consecutive iteration ranges of it
    assert d["measured"] is True
    assert len(d["step_s"]) == d["steps"] and abs(sum(d["step_s"]) - d["value"]) < 0.01 + 1e-3 * d["value"]
    assert d["timed_region_s"] == d["value"] and d["max_true_residual"] <= 1e-10 * 1.01
    assert d["config"]["workload"].startswith("c1: 1000 rows")


def test_reference_arm_splits_one_solve_into_steps():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "c1", "--scale", "12",
                        "--steps", "5", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    (d,) = _json_lines(r.stdout)
    assert d["steps"] == 5 and len(d["step_s"]) == 5 and all(t >= 0 for t in d["step_s"])
    assert abs(sum(d["step_s"]) - d["value"]) < 0.01 + 1e-3 * d["value"]
    assert abs(d["ms_per_step"] - d["value"] * 1e3 / 5) < 1e-6 * d["value"] * 1e3


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


def test_clock_summary_reads_nvidia_smi_lines():
    """The clocks object of a bench line: median SM clock under load, the
    maximum, and every throttle reason seen active in any sample."""
    sys.path.insert(0, str(ROOT))
    import bench

    c = bench.Clocks(0)
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1995, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 1800, 2070, 1400.0, 0x0000000000000008, Active, Not Active, Not Active, Active",
        "garbage line",
        "0, [N/A], 2070, 1.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = c.summary()
    assert s["sm_mhz"] == 1995.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert bench.Clocks(0).summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
