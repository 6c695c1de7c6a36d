"""Replicas across processes (slam_gb300.distributed) on the CPU with the
gloo backend, two ranks: the pair shares cover every pair once, the host
gather restores pair order, and the whole-job rate uses the slowest rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from slam_gb300 import distributed


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_covers_every_pair_once():
    for n in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            got = []
            for r in range(world):
                b, e = distributed.shard(n, r, world)
                got.extend(range(b, e))
            assert got == list(range(n)), (n, world)
            sizes = [e - b for b, e in (distributed.shard(n, r, world) for r in range(world))]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        distributed.shard(4, 2, 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 11
        b, e = distributed.shard(n, rank, world)
        local = [i * i for i in range(b, e)]          # a per-pair result of this rank's share
        full = distributed.gather_results(local)
        slowest = distributed.max_over_ranks(1.0 + rank)
        rate = distributed.job_rate(e - b, 1.0 + rank)
        q.put((rank, full, slowest, rate))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_ranks_gather_and_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, full, slowest, rate in out:
        assert full == [i * i for i in range(11)]
        assert slowest == 2.0                          # the slower rank's time
    rates = sorted(r for _, _, _, r in out)
    # each rank reports world x its own units over the slowest time: 2 x 6 / 2 and 2 x 5 / 2
    assert rates == [5.0, 6.0]


def test_single_process_identity():
    assert distributed.gather_results([1, 2]) == [1, 2]
    assert distributed.max_over_ranks(3.5) == 3.5
    assert distributed.job_rate(10, 2.0) == 5.0
