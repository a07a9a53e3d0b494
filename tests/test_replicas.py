"""The multi-GPU path of bench.py is replicas only: every rank advances its
own scene and the whole-job rate is the units of all ranks over the slowest
rank's time.  Checked here with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, out) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(REPO))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        units = 1000.0 * (rank + 1)
        seconds = 0.5 + rank  # rank 1 is the slow one
        out.put((rank, bench.replica_rate(units, seconds, dist, "cpu")))
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        rate, slowest = results[r]
        assert slowest == pytest.approx(1.5)
        assert rate == pytest.approx(3000.0 / 1.5)


def _rank_teardown(rank: int, world: int, port: int, out) -> None:
    """A rank's end as bench.py's GPU arm ends it: the whole-job rate, then
    finish_rank (simulation closed, process group destroyed once)."""
    import torch.distributed as dist
    sys.path.insert(0, str(REPO))
    import bench

    class _Sim:
        closed = 0

        def close(self):
            _Sim.closed += 1

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    rate, _ = bench.replica_rate(10.0, 1.0, dist, "cpu")
    sim = _Sim()
    bench.finish_rank(sim, dist)
    out.put((rank, rate, _Sim.closed, dist.is_initialized()))


def test_teardown_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_teardown, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = {r: (rate, closed, live) for r, rate, closed, live in (q.get(timeout=120) for _ in range(2))}
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0, "a rank failed in its teardown"
    for r in range(2):
        rate, closed, live = results[r]
        assert rate == pytest.approx(20.0) and closed == 1 and not live


def test_replica_rate_single_process():
    sys.path.insert(0, str(REPO))
    import bench
    assert bench.replica_rate(100.0, 2.0) == (50.0, 2.0)
