"""Multi-GPU without a data-path collective.

A frame does not shard without redoing its geometry on every GPU, but independent frames and
views do: each rank renders its own frames (replicas) or its share of a batch's views, and the
only communication is the host-side bookkeeping below (timing and unit counts, over whatever
process group the caller set up: NCCL on GPUs, gloo on CPUs).
"""


def shard(n_items, rank, world):
    """The contiguous, balanced range of item indices that `rank` of `world` owns (the first
    n_items % world ranks take one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def job_time(seconds, dist=None, device=None):
    """The whole job's time: the maximum over ranks of each rank's time (the slowest rank ends the
    job). Without a process group, the local time."""
    if dist is None:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def total_units(units, dist=None, device=None):
    """Units (triangles, pixels, views) processed by all ranks together."""
    if dist is None:
        return int(units)
    import torch
    t = torch.tensor([int(units)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def throughput(units, seconds, dist=None, device=None):
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    return total_units(units, dist, device) / job_time(seconds, dist, device)
