"""HBM brick pool residency: the reference cache's LRU semantics
(livre/core/cache/Cache.cpp:41-209, tests/core/cache.cpp:29-78), ancestor
fallback of the asynchronous mode (RenderingSetGeneratorFilter.cpp:32-111)
and the bytes streamed through data-source callbacks."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_ctx(n_slots, vi):
    """A context whose pool holds n_slots bricks of volume vi."""
    import livre_gb300 as lv
    return lv.Context(0, pool_bytes=n_slots * vi.slot_bytes)


def test_cache_known_answer():
    """tests/core/cache.cpp: budget of 2 objects; load 1, 2, 1 (hit, no
    refresh), 3 -> 1 is evicted; purge empties the cache."""
    import livre_gb300 as lv
    vol = lv.VolumeInformation(64, 16, 1)
    ctx = small_ctx(2, vol)
    v = ctx.blob_volume(vol, 4, 1)
    a, b, c = (lv.NodeId(1, p).id for p in [(0, 0, 0), (0, 0, 1), (0, 1, 0)])
    assert v.load([a]) == 1
    assert v.load([b]) == 1
    assert v.resident() == [a, b]
    assert v.load([a]) == 0          # hit
    assert v.resident() == [a, b]    # order unchanged
    assert v.load([c]) == 1
    assert v.resident() == [b, c]
    ctx.purge()
    assert v.resident() == []
    v.close()
    ctx.close()


def test_eviction_skips_bricks_in_use(oracle):
    """A frame whose visible set fills the pool evicts only bricks it does not use."""
    import livre_gb300 as lv
    vol = lv.VolumeInformation(128, 32, 1)
    ovol = oracle.volume(128, 32, 1)
    mv, proj = lv.orbit_camera(0, 8, vol.world_size, 64, 64, radius_scale=1.0)
    vis, _ = oracle.select_visible(ovol, mv, proj, 64, 1.0)
    vis = [int(i) for i in vis]
    ctx = small_ctx(len(vis) + 3, vol)
    v = ctx.blob_volume(vol, 6, 2)
    others = [n.id for n in vol.all_nodes() if n.id not in set(vis)][:5]
    assert v.load(others) == 5
    tf = ctx.transfer_function(lv.linear_ramp_tf())
    desc = ctx.render_desc(mv, proj, 64, 64, sse=1.0)
    ctx.render(v, tf, desc)
    st = ctx.last_stats()
    assert st["n_available"] == len(vis) and st["n_not_available"] == 0
    res = v.resident()
    # the two oldest of `others` made room; everything visible is resident
    assert set(vis) <= set(res)
    assert res[:3] == others[2:]
    v.close()
    ctx.close()


def expected_rendering_set(visible, resident):
    """RenderingSetGenerator (RenderingSetGeneratorFilter.cpp:32-111) in Python."""
    import livre_gb300 as lv
    res = set(resident)
    chosen = {}
    for i in visible:
        n = lv.NodeId(i)
        while n.is_valid():
            if n.id in res:
                chosen[n.id] = True
                break
            n = n.get_parent()
    out = set()
    for i in chosen:
        if not any(p.id in chosen for p in lv.NodeId(i).get_parents()):
            out.add(i)
    return sorted(out)


def test_async_ancestor_fallback(oracle):
    import livre_gb300 as lv
    vol = lv.VolumeInformation(128, 32, 1)
    ovol = oracle.volume(128, 32, 1)
    ctx = lv.Context(0, pool_bytes=256 << 20)
    v = ctx.blob_volume(vol, 10, 5)
    tf_rgba = lv.linear_ramp_tf()
    tf = ctx.transfer_function(tf_rgba)
    mv, proj = lv.orbit_camera(1, 8, vol.world_size, 64, 48, radius_scale=1.1)
    vis, _ = oracle.select_visible(ovol, mv, proj, 48, 1.0)
    v.load([lv.NodeId(0, (0, 0, 0)).id])  # only the root is resident
    bp = oracle.blob_params(10, 5, 0, 1)
    seen_complete = False
    for frame in range(40):
        desc = ctx.render_desc(mv, proj, 64, 48, sse=1.0, synchronous=False, max_uploads=3)
        img = ctx.render(v, tf, desc).cpu().numpy()
        st = ctx.last_stats()
        # uploads of the previous frame's misses happen before this frame resolves
        want = expected_rendering_set(vis, v.resident())
        assert st["n_rendered"] == len(want)
        assert st["n_available"] + st["n_not_available"] == len(vis)
        bricks = np.stack([oracle.blob_brick(ovol, bp, i) for i in want])
        view = oracle.make_view(mv, proj, 64, 48, st["samples_per_ray"])
        ref, _ = oracle.raycast(ovol, 1, want, bricks, tf_rgba, view)
        assert np.abs(img - ref).max() <= 1.0 / 255.0
        if st["n_not_available"] == 0:
            seen_complete = True
            break
    assert seen_complete
    v.close()
    ctx.close()


def test_callback_source_bytes():
    """A DataSourcePlugin-style callback fills pinned staging; the volume's
    bricks are what the callback wrote (mem:// constant bricks,
    livre/data/MemoryDataSource.cpp:38-61)."""
    import livre_gb300 as lv
    import math
    vol = lv.VolumeInformation(64, 16, 1)
    calls = []

    def get_data(node_id, dst, nbytes):
        calls.append(node_id)
        b = node_id.to_bytes(8, "little")
        value = (b[0] ^ b[1] ^ b[2] ^ b[3]) + 16 + int(127 * math.sin(1 / 200.0))
        ctypes.memset(dst, value & 0xFF, nbytes)
        return True

    ctx = lv.Context(0, pool_bytes=64 << 20)
    v = ctx.callback_volume(vol, get_data)
    ids = [lv.NodeId(1, (1, 0, 1)).id, lv.NodeId(0, (0, 0, 0)).id]
    assert v.load(ids) == 2
    assert calls == ids
    tf = ctx.transfer_function(lv.linear_ramp_tf())
    mv, proj = lv.orbit_camera(0, 8, vol.world_size, 32, 32)
    ctx.render(v, tf, ctx.render_desc(mv, proj, 32, 32, sse=8.0, max_lod=0))
    st = ctx.last_stats()
    assert st["n_uploaded"] == 0 and st["n_rendered"] == 1
    v.close()
    ctx.close()
