"""Multi-GPU rendering, one process per GPU.

Replicas: views are independent, so the render path shards by view index
with no data-path collective (the reference distributes channels through
Equalizer, livre/eq/Channel.cpp:234-281, which is not rebuilt): rank r
renders views r, r + N, r + 2N, ... . The only exchange is timing: the job
time is the maximum over ranks and the job rate counts every rank's views.

Sort-first bands: one frame split into N horizontal bands of rows (the
reference's sort-first tiles, Channel.cpp:234-281), rank r ray casting band r
(lv_render_desc.rect) with the whole frame's visible set, and the bands
gathered to one frame through host memory. The stitched frame equals the
frame rendered whole, bit for bit.
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


def band(height, rank, world):
    """Rows (y0, rows) of band `rank` of `world`: near-equal consecutive
    bands from row 0 up, the first height % world one row taller."""
    base, extra = divmod(int(height), int(world))
    y0 = rank * base + min(rank, extra)
    return y0, base + (1 if rank < extra else 0)


def gather_bands(frame, dist, world, rank, dst=0):
    """Stitches every rank's band of an (H, W, C) frame into rank `dst`'s
    `frame` through host memory (a gather of the host copies of the bands;
    the other ranks' frames are left as they are). Works with any backend
    that gathers CPU tensors (gloo)."""
    import torch
    H = frame.shape[0]
    y0, rows = band(H, rank, world)
    mine = frame[y0:y0 + rows].contiguous().cpu()
    if dist is None or world == 1:
        return frame
    tallest = band(H, 0, world)[1]
    padded = torch.zeros((tallest,) + tuple(frame.shape[1:]), dtype=frame.dtype)
    padded[:rows] = mine
    parts = [torch.zeros_like(padded) for _ in range(world)] if rank == dst else None
    dist.gather(padded, parts, dst=dst)
    if rank == dst:
        for r, part in enumerate(parts):
            ry0, rrows = band(H, r, world)
            frame[ry0:ry0 + rrows] = part[:rrows].to(frame.device)
    return frame
