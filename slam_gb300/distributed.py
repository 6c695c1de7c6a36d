"""Multi-GPU use of the tracker: replicas, one process per GPU.

A single tracking call is one sequential Gauss-Newton problem and does not
shard; many independent frame pairs (loop-closure candidates, the batched
verification workload) shard by pair index with no data-path collective.
These helpers cover the host side: the contiguous share of pairs of a rank,
the gather of per-pair results on the host, and the whole-job timing (the
slowest rank's time, every rank's work)."""


def shard(n, rank, world):
    """[begin, end) of the pairs rank `rank` of `world` tracks: contiguous
    shares whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard request (n=%d, rank=%d, world=%d)" % (n, rank, world))
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def gather_results(local):
    """Every rank's list of per-pair results (picklable), concatenated in
    rank order = pair order for shard(); the identity without a process
    group."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return list(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, list(local))
    return [r for p in parts for r in p]


def max_over_ranks(value):
    """The largest of the ranks' values (a timed region's duration: the job
    ends with its slowest rank)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch
    backend = dist.get_backend()
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device="cuda" if backend == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, seconds_per_rank):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    dist = _dist()
    world = 1 if dist is None else dist.get_world_size()
    return world * units_per_rank / max_over_ranks(seconds_per_rank)

