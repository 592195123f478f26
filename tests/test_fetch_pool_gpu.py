"""Host fetch threads of callback sources (lv_volume_set_fetch_threads).

Bricks fetched by several host threads at once must land in the pool exactly
as with one fetching thread: the same bytes, each missing brick fetched once,
null bricks skipped (DataUploadFilter.cpp:56-64), and identical frames.
"""
import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    c = lv.Context(0, pool_bytes=512 << 20)
    yield c
    c.close()


def _render(ctx, vol, tf, info, k=1):
    import livre_gb300 as lv
    mv, proj = lv.orbit_camera(k, 8, info.world_size, 128, 96, radius_scale=1.1)
    img = ctx.render(vol, tf, ctx.render_desc(mv, proj, 128, 96, sse=1.0)).cpu().numpy()
    return img, ctx.last_stats()


@pytest.mark.parametrize("threads", [1, 3, 8, 0])
def test_fbm_host_volume_same_frame_any_thread_count(ctx, threads):
    import livre_gb300 as lv
    info = lv.VolumeInformation(256, 32, overlap=1, dtype=lv.DT_UINT16)
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=2))
    dev = ctx.fbm_volume(info, 5, placement=lv.FBM_DEVICE)
    want, st_dev = _render(ctx, dev, tf, info)
    dev.close()
    ctx.purge()
    host = ctx.fbm_volume(info, 5, placement=lv.FBM_HOST, host_threads=threads)
    if threads:
        assert host.fetch_threads == threads
    else:
        assert 1 <= host.fetch_threads <= 64
    got, st = _render(ctx, host, tf, info)
    assert st["n_uploaded"] == st_dev["n_uploaded"] == st["n_rendered"] > 8
    np.testing.assert_array_equal(got, want)  # same bytes in the pool
    for nid in host.resident()[:4]:
        np.testing.assert_array_equal(host.get_data(nid), lv.fbm_brick(info, nid, 5))
    host.close()
    tf.close()


def test_reentrant_callback_fetched_once_per_brick(ctx):
    import livre_gb300 as lv
    info = lv.VolumeInformation(192, 32, overlap=1, dtype=lv.DT_UINT8)
    calls, lock, threads_seen = [], threading.Lock(), set()

    def get_data(node_id, dst, nbytes):
        with lock:
            calls.append(node_id)
            threads_seen.add(threading.get_ident())
        if lv.NodeId(node_id).position[0] == 1:
            return False  # a null MemoryUnitPtr: the brick is skipped
        value = 16 + (node_id * 2654435761 >> 7) % 200
        C.memset(dst, int(value), nbytes)
        return True

    tf = ctx.transfer_function(lv.linear_ramp_tf(256))
    frames = {}
    for n in (1, 4):
        ctx.purge()
        calls.clear()
        vol = ctx.callback_volume(info, get_data)
        vol.fetch_threads = n
        img, st = _render(ctx, vol, tf, info, k=2)
        assert len(calls) == len(set(calls)) == st["n_visible"]  # once each
        skipped = sum(1 for c in calls if lv.NodeId(c).position[0] == 1)
        assert skipped > 0 and st["n_uploaded"] == len(calls) - skipped
        resident = vol.resident()
        assert all(lv.NodeId(r).position[0] != 1 for r in resident)
        frames[n] = img
        vol.close()
    np.testing.assert_array_equal(frames[1], frames[4])
    tf.close()


def test_fetch_threads_validation(ctx):
    import livre_gb300 as lv
    info = lv.VolumeInformation(64, 32, overlap=1)
    blob = ctx.blob_volume(info, 4, seed=1)
    with pytest.raises(lv.LivreError):
        blob.fetch_threads = 4  # generated on the device: nothing to fetch
    vol = ctx.callback_volume(info, lambda n, d, b: True)
    assert vol.fetch_threads == 1
    with pytest.raises(lv.LivreError):
        vol.fetch_threads = 65
    vol.fetch_threads = 0  # one per hardware thread, at most 64
    assert 1 <= vol.fetch_threads <= 64
    vol.close()
    blob.close()
