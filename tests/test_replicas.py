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
