"""lv_select_visible_noalloc: the LOD selection for callers that cannot
allocate device memory (for example a host application whose own allocator
owns the GPU's memory). Called through the C ABI, its output must equal
lv_select_visible's (NodeIds are integers: exact equality) on two calls in a
row, since every call reuses the same fixed device scratch.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_noalloc(native, abi, vol, cam, lod, out, res):
    import torch
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = native.lv_select_visible_noalloc(C.byref(vol.info), C.byref(cam), C.byref(lod),
                                          C.c_void_p(out.data_ptr()), out.numel(),
                                          C.c_void_p(res.data_ptr()), stream)
    assert st == abi.LV_OK, st
    torch.cuda.synchronize()
    r = res.cpu().numpy().view(np.uint32).copy()
    return np.sort(out[: r[abi.SEL_WRITTEN]].cpu().numpy().view(np.uint64)), r


def test_noalloc_matches_select_visible(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    from livre_gb300 import _abi
    ctx = lv.Context(0, pool_bytes=64 << 20)
    vol = lv.VolumeInformation(2048, 64, 1)
    out = torch.empty(vol.node_count(), dtype=torch.int64, device="cuda")
    res = torch.zeros(_abi.SELECT_RESULT_WORDS, dtype=torch.int32, device="cuda")
    for k, (sse, H) in enumerate([(1.0, 1080), (0.5, 2160)]):  # two calls in a row
        mv, proj = lv.orbit_camera(3 + 5 * k, 16, vol.world_size, 1920, H, radius_scale=0.9)
        cam, lod = lv.make_camera(mv, proj), lv.make_lod(H, sse)
        got, r = _call_noalloc(native, _abi, vol, cam, lod, out, res)
        want, wr = ctx.select_visible(vol, mv, proj, H, sse)
        assert len(got) > 8
        assert got.tolist() == sorted(want.tolist())
        assert r[_abi.SEL_VISITED] == wr[_abi.SEL_VISITED]
        assert r[_abi.SEL_MAX_LEVEL] == wr[_abi.SEL_MAX_LEVEL]
        assert r[_abi.SEL_OVERFLOW] == 0
    ctx.close()


def test_noalloc_capacity_lod_limits_and_clip(native):
    """The parameters the no-allocation call takes apart from the view: a
    capacity below the visible count (WRITTEN clamped, FOUND the full
    count), minimum / maximum LOD and a clip plane, each equal to
    lv_select_visible's result."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    from livre_gb300 import _abi
    ctx = lv.Context(0, pool_bytes=64 << 20)
    vol = lv.VolumeInformation(1024, 32, 1)
    mv, proj = lv.orbit_camera(5, 16, vol.world_size, 1280, 720, radius_scale=0.8)
    res = torch.zeros(_abi.SELECT_RESULT_WORDS, dtype=torch.int32, device="cuda")
    # capacity below the visible count
    want, wr = ctx.select_visible(vol, mv, proj, 720, 1.0)
    assert wr[_abi.SEL_FOUND] > 16
    small = torch.empty(16, dtype=torch.int64, device="cuda")
    got, r = _call_noalloc(native, _abi, vol, lv.make_camera(mv, proj), lv.make_lod(720, 1.0),
                           small, res)
    assert r[_abi.SEL_WRITTEN] == 16 and len(got) == 16
    assert r[_abi.SEL_FOUND] == wr[_abi.SEL_FOUND]
    assert set(got.tolist()) <= set(want.tolist())
    # LOD limits and a clip plane
    out = torch.empty(vol.node_count(), dtype=torch.int64, device="cuda")
    clip = [(0.3, 1.0, -0.2, 0.05)]
    for min_lod, max_lod in [(2, 3), (0, 1), (3, 3)]:
        lod = lv.make_lod(720, 1.0, min_lod, max_lod, clip_planes=clip)
        got, r = _call_noalloc(native, _abi, vol, lv.make_camera(mv, proj), lod, out, res)
        want, wr = ctx.select_visible(vol, mv, proj, 720, 1.0, min_lod, max_lod,
                                      clip_planes=clip)
        assert len(got) > 0
        assert got.tolist() == sorted(want.tolist()), (min_lod, max_lod)
        assert r[_abi.SEL_FOUND] == wr[_abi.SEL_FOUND]
        assert r[_abi.SEL_VISITED] == wr[_abi.SEL_VISITED]
        assert r[_abi.SEL_MAX_LEVEL] == wr[_abi.SEL_MAX_LEVEL]
    ctx.close()


def test_noalloc_rejects_oversized_volume(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    from livre_gb300 import _abi
    big = lv.VolumeInformation(16384, 64, 1)  # 2^21 nodes in its finest level
    mv, proj = lv.orbit_camera(0, 8, big.world_size, 64, 64)
    out = torch.empty(16, dtype=torch.int64, device="cuda")
    res = torch.zeros(_abi.SELECT_RESULT_WORDS, dtype=torch.int32, device="cuda")
    st = native.lv_select_visible_noalloc(C.byref(big.info), C.byref(lv.make_camera(mv, proj)),
                                          C.byref(lv.make_lod(64, 1.0)),
                                          C.c_void_p(out.data_ptr()), 16,
                                          C.c_void_p(res.data_ptr()), None)
    assert st == _abi.LV_ENOMEM
    lod = lv.make_lod(64, 1.0, rng=(0.0, 0.5))
    small = lv.VolumeInformation(256, 32, 1)
    st = native.lv_select_visible_noalloc(C.byref(small.info), C.byref(lv.make_camera(mv, proj)),
                                          C.byref(lod), C.c_void_p(out.data_ptr()), 16,
                                          C.c_void_p(res.data_ptr()), None)
    assert st == _abi.LV_EINVAL
