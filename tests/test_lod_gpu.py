"""Device LOD selection (lv_select_visible) against the reference's golden ids
and, bit-exactly, against the oracle on random cameras."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("case", range(8))
def test_golden_lod_selection_gpu(gpu_ctx, case):
    import livre_gb300 as lv
    g = json.load(open(os.path.join(GOLDEN, "lod_selection.json")))
    c = g["cases"][case]
    vol = lv.VolumeInformation(4096, 256, 4)
    ids, res = gpu_ctx.select_visible(vol, g["mv"], g["proj"], c["window_height"], c["sse"],
                                      c["min_lod"], c["max_lod"])
    assert sorted(int(i) for i in ids) == c["expected"]
    assert res[lv._abi.SEL_OVERFLOW] == 0


def random_camera(rng, world, inside=False):
    import livre_gb300 as lv
    diag = float(np.linalg.norm(world))
    if inside:
        eye = rng.uniform(-0.45, 0.45, 3) * np.array(world)
        target = rng.uniform(-0.5, 0.5, 3)
        near = 0.01
    else:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        eye = d * rng.uniform(0.8, 3.0) * diag
        target = rng.uniform(-0.2, 0.2, 3)
        near = 0.1
    if np.linalg.norm(target - eye) < 1e-3:
        target = eye + np.array([0.0, 0.0, -1.0])
    up = (0.0, 1.0, 0.0) if abs((target - eye)[1]) < 0.99 * np.linalg.norm(target - eye) else (1, 0, 0)
    fov = rng.uniform(30, 70)
    aspect = rng.uniform(0.5, 2.0)
    return lv.look_at(eye, target, up), lv.perspective(fov, aspect, near, 15.0)


VOLUMES = [((256, 256, 256), 32, 1), ((2048, 2048, 2048), 64, 1), ((2048, 2099, 2048), 64, 0),
           ((1024, 1024, 512), 32, 4), ((8192, 8192, 8192), 128, 1)]


@pytest.mark.parametrize("vi", range(len(VOLUMES)))
def test_random_cameras_bit_exact(gpu_ctx, oracle, vi):
    import livre_gb300 as lv
    voxels, block, overlap = VOLUMES[vi]
    vol = lv.VolumeInformation(voxels, block, overlap)
    ovol = oracle.volume(voxels, block, overlap)
    rng = np.random.default_rng(100 + vi)
    for trial in range(12):
        mv, proj = random_camera(rng, vol.world_size, inside=trial % 3 == 2)
        H = int(rng.choice([256, 512, 1080, 2160]))
        sse = float(rng.uniform(0.5, 4.0))
        min_lod = int(rng.integers(0, 2))
        max_lod = int(rng.choice([100, vol.depth - 2 if vol.depth > 2 else 0]))
        want, visited = oracle.select_visible(ovol, mv, proj, H, sse, min_lod, max_lod)
        got, res = gpu_ctx.select_visible(vol, mv, proj, H, sse, min_lod, max_lod)
        assert sorted(got.tolist()) == sorted(want.tolist()), (vi, trial)
        assert res[lv._abi.SEL_VISITED] == visited
        if len(want):
            assert res[lv._abi.SEL_MAX_LEVEL] == max(int(i) & 0xF for i in want)


def test_clip_planes_and_time_step(gpu_ctx, oracle):
    import livre_gb300 as lv
    vol = lv.VolumeInformation(512, 32, 1)
    ovol = oracle.volume(512, 32, 1)
    mv, proj = lv.orbit_camera(3, 16, vol.world_size, 800, 600)
    planes = [(1.0, 0.0, 0.0, 0.1), (0.0, -0.7071, 0.7071, 0.2)]
    want, _ = oracle.select_visible(ovol, mv, proj, 600, 1.0, clip_planes=planes, time_step=7)
    got, _ = gpu_ctx.select_visible(vol, mv, proj, 600, 1.0, clip_planes=planes, time_step=7)
    assert sorted(got.tolist()) == sorted(want.tolist())
    assert all((int(i) >> 46) == 7 for i in got)


@pytest.mark.parametrize("rng_", [(0.0, 0.5), (0.25, 0.75), (0.5, 1.0), (0.1, 0.1)])
def test_sort_last_range_slice(gpu_ctx, oracle, rng_):
    """visitPost keeps DFS indices [start, end) (SelectVisibles.cpp:110-131)."""
    import livre_gb300 as lv
    vol = lv.VolumeInformation(1024, 32, 1)
    ovol = oracle.volume(1024, 32, 1)
    mv, proj = lv.orbit_camera(1, 8, vol.world_size, 1024, 768)
    want, _ = oracle.select_visible(ovol, mv, proj, 768, 1.0, rng=rng_)
    got, _ = gpu_ctx.select_visible(vol, mv, proj, 768, 1.0, rng=rng_)
    # the slice is in DFS order on both sides
    assert got.tolist() == want.tolist()


def test_capacity_overflow_reported(gpu_ctx):
    import torch
    import livre_gb300 as lv
    vol = lv.VolumeInformation(1024, 32, 1)
    mv, proj = lv.orbit_camera(0, 8, vol.world_size, 1024, 1024, radius_scale=0.9)
    out = torch.empty(4, dtype=torch.int64, device="cuda")
    o, res = gpu_ctx.select_visible(vol, mv, proj, 1024, 0.5, out=out)
    assert res[lv._abi.SEL_FOUND] > 4 and res[lv._abi.SEL_WRITTEN] == 4
