"""bench.py's multi-rank plumbing (replicas, no data exchange) on CPU with
two gloo ranks: barrier, max of per-rank times, sum of per-rank work."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    r = bench.Ranks()
    r.barrier()
    t = r.reduce(1.0 + rank, "max")
    units = r.reduce(10.0 * (rank + 1), "sum")
    r.barrier()
    r.close()
    q.put((rank, t, units))


def test_two_rank_max_and_sum():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_reference_arm_only_rank0_prints(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    class FakeRanks:
        rank, world = 1, 2

    assert bench.run_reference(type("A", (), {"workload": "jet_d3q27", "warmup": 1, "steps": 1})(), FakeRanks()) is None
