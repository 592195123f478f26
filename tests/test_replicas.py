"""Replicas across ranks (the multi-GPU form of the path): views shard by
index with no data-path collective, timing is the maximum over ranks. Two
gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from livre_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(64, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        times = replicas.max_over_ranks([1.0 + rank, 10.0 - rank], dist)
        out[rank] = (gathered, times, replicas.job_rate(len(mine), world, times[0]))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas():
    import torch.multiprocessing as mp
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    gathered = res[0][0]
    assert sorted(i for part in gathered for i in part) == list(range(64))
    assert not set(gathered[0]) & set(gathered[1])
    for r in range(world):
        assert res[r][1] == [2.0, 10.0]      # max over ranks, element-wise
        assert res[r][2] == pytest.approx(64 / 2.0)


def test_shard_edges():
    from livre_gb300 import replicas
    assert replicas.shard(3, 5, 8) == [2]    # more ranks than views: still one view
    assert replicas.shard(0, 0, 2) == [0]
    assert replicas.max_over_ranks([1.5]) == [1.5]


def _band_rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from livre_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        H, W = 37, 5
        # each rank "renders" its band: the rows it owns get frame values,
        # the rest a marker the gather must overwrite
        full = torch.arange(H * W * 4, dtype=torch.float32).reshape(H, W, 4)
        frame = torch.full((H, W, 4), -1.0)
        y0, rows = replicas.band(H, rank, world)
        frame[y0:y0 + rows] = full[y0:y0 + rows]
        replicas.gather_bands(frame, dist, world, rank, dst=0)
        out[rank] = (frame.tolist(), full.tolist())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sort_first_bands_gather_to_the_whole_frame(world):
    import torch.multiprocessing as mp
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_band_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    frame, full = res[0]
    assert frame == full
    for r in range(1, world):
        assert res[r][0] != full  # only the destination is stitched


def test_band_partition():
    from livre_gb300 import replicas
    for H in (1, 2, 7, 1080, 2160):
        for world in (1, 2, 3, 4, 8):
            bands = [replicas.band(H, r, world) for r in range(world)]
            assert bands[0][0] == 0
            assert all(a[0] + a[1] == b[0] for a, b in zip(bands, bands[1:]))
            assert bands[-1][0] + bands[-1][1] == H
            assert max(b[1] for b in bands) - min(b[1] for b in bands) <= 1
