"""Replicated rendering, one process per GPU.

Views are independent, so the render path shards by view index with no
data-path collective (the reference distributes channels through Equalizer,
livre/eq/Channel.cpp:234-281, which is not rebuilt): rank r renders views
r, r + N, r + 2N, ... . The only exchange is timing: the job time is the
maximum over ranks and the job rate counts every rank's views.
"""


def shard(n_items, rank, world):
    """Indices of the items rank `rank` of `world` renders (at least one)."""
    mine = [k for k in range(n_items) if k % world == rank]
    return mine or [rank % max(n_items, 1)]


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return units_per_rank * world / seconds
