"""bench.py --gpus N runs N independent replicas (a batch of problems shards
with no data-path exchange). Its whole-job figures take each time's maximum
over the ranks and divide all ranks' solves by it; this checks that logic
with two gloo ranks on the CPU."""

from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 10 + r ms for its 8 solves, and 2 + 3r s for a batch of 4096
        got = bench.replica_max([10.0 + rank, 2.0 + 3.0 * rank], world, "cpu")
        q.put((rank, got, bench.job_ms_per_solve(got[0], 1, 8, world), bench.job_solves_per_s(got[1], 4096, world)))
    finally:
        dist.destroy_process_group()


def test_replica_figures_take_the_slowest_rank_over_all_solves() -> None:
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    world, port = 2, _free_port()
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, ms_per_solve, solves_per_s in out:
        assert got == [11.0, 5.0]  # every rank sees the slowest rank's times
        assert ms_per_solve == pytest.approx(11.0 / 16)  # 16 solves in all, in the slowest rank's 11 ms
        assert solves_per_s == pytest.approx(2 * 4096 / 5.0)


def test_single_replica_is_unchanged() -> None:
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_max([3.0, 4.5], 1, "cpu") == [3.0, 4.5]
    assert bench.job_ms_per_solve(80.0, 2, 8, 1) == pytest.approx(5.0)
    assert bench.job_solves_per_s(0.5, 4096, 1) == pytest.approx(8192.0)
