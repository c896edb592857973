"""Multi-rank host logic of bench.py on CPU: gloo, world size 2.

The GPU path runs one replica of the whole workload per rank (the shells of a
step never exchange data); what crosses ranks is the barrier around the timed
region and the max-over-ranks of its duration.  These run as two CPU
processes over gloo on 127.0.0.1.
"""

from __future__ import annotations

import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        dist.barrier()
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")
        value = bench.job_value(world, 40, ms / 5)
        # the reference arm: rank 0 alone runs and prints, the others return nothing
        class A:
            steps, warmup, cpu_shells, nside, nshell, lmax = 1, 0, 0, 8, 2, 8
        ref = bench.run_reference(A, rank, world) if rank != 0 else "rank0"
        out.put((rank, ms, value, ref))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]  # both ranks see the slowest rank's time
    assert res[0][2] == pytest.approx(2 * 40 / (4.0 / 1e3))  # all ranks' shells / max time
    assert res[1][3] is None  # rank 1 of the reference arm does no work


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.job_value(1, 40, 80.0) == pytest.approx(500.0)
