"""The multi-GPU host path of bench.py (replicas: one rank per GPU, no
collective on the data path) on CPU: two gloo ranks agree on the whole-job step
time (max over ranks) and the work done (sum over ranks)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, str(ROOT))
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    d = bench.Dist(backend="gloo")
    try:
        d.barrier()
        step, units = bench.aggregate(d, 1.0 + rank, 2.0 + rank)
        out.put((rank, step, units))
    finally:
        d.close()


@pytest.mark.parametrize("world", [2])
def test_replica_aggregation_over_gloo(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, step, units in got:
        assert step == float(world)  # max over ranks of 1 + rank
        assert units == sum(2.0 + r for r in range(world))


def test_single_rank_is_identity():
    import sys

    sys.path.insert(0, str(ROOT))
    import bench

    for key in ("WORLD_SIZE", "RANK"):
        os.environ.pop(key, None)
    d = bench.Dist()
    assert d.world == 1 and bench.aggregate(d, 3.5, 1.0) == (3.5, 1.0)
