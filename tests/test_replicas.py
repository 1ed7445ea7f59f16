"""Replicas across processes (the multi-GPU mode of the path), on CPU with
gloo and world size 2: every unit is reconstructed by exactly one rank and
the job's time is the slowest rank's."""
import os
import socket

import pytest

from fastrecon_gb300 import replicas


def test_shard_covers_every_unit_once():
    for n in (0, 1, 5, 8, 64, 1001):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = replicas.shard(n, r, world)
                assert 0 <= lo <= hi <= n
                seen.extend(range(lo, hi))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = replicas.shard(10, rank, world)
        elapsed = 1.0 + rank  # rank 1 is the slower one
        job = replicas.max_over_ranks(elapsed, dist)
        units = replicas.sum_over_ranks(hi - lo, dist)
        dist.barrier()
        out.put((rank, lo, hi, job, units))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_units_and_report_the_slowest():
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
    (r0, lo0, hi0, job0, n0), (r1, lo1, hi1, job1, n1) = res
    assert (lo0, hi0, lo1, hi1) == (0, 5, 5, 10)
    assert job0 == job1 == 2.0
    assert n0 == n1 == 10
