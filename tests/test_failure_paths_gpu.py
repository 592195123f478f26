"""Failure paths the runtime handles, made to happen without faulting the
GPU (bounded waits that run out, exceptions thrown on the host).

- The single-view selection's cooperative launch waits at a grid barrier;
  every wait is bounded. lv_test_fail_grid_barrier makes one CTA of the next
  such launch skip the barrier and shortens the bound: the other CTAs give
  up, the launch returns, the selection reports LV_SEL_OVERFLOW = 2, and the
  context renders and selects correctly afterwards.
- A data-source plugin whose getData throws (tests/plugins/flaky_source.cpp):
  the brick is skipped as for a null MemoryUnitPtr
  (DataUploadFilter.cpp:56-64), the frame completes, and it equals the frame
  of the same volume served by a callback returning no data for those
  bricks. A getData that sleeps delays its brick but the frame still gets it.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_grid_barrier_timeout_reported(gpu_ctx, native):
    import livre_gb300 as lv
    from livre_gb300 import _abi
    vol = lv.VolumeInformation(2048, 64, 1)
    mv, proj = lv.orbit_camera(1, 8, vol.world_size, 1920, 1080)
    want, wr = gpu_ctx.select_visible(vol, mv, proj, 1080, 1.0)
    assert wr[_abi.SEL_OVERFLOW] == 0 and len(want) > 8
    with pytest.raises(lv.LivreError):
        lv.check(native.lv_test_fail_grid_barrier(gpu_ctx.handle, 0), gpu_ctx.handle)
    lv.check(native.lv_test_fail_grid_barrier(gpu_ctx.handle, 2000), gpu_ctx.handle)
    _, r = gpu_ctx.select_visible(vol, mv, proj, 1080, 1.0)
    assert r[_abi.SEL_OVERFLOW] == 2  # a barrier wait gave up
    # the hook is spent and the context is usable
    again, r2 = gpu_ctx.select_visible(vol, mv, proj, 1080, 1.0)
    assert r2[_abi.SEL_OVERFLOW] == 0
    assert sorted(again.tolist()) == sorted(want.tolist())
    v = gpu_ctx.blob_volume(lv.VolumeInformation(128, 32, 1), 8, seed=1)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf(256))
    m2, p2 = lv.orbit_camera(2, 8, (1.0, 1.0, 1.0), 64, 64, radius_scale=1.2)
    gpu_ctx.render(v, tf, gpu_ctx.render_desc(m2, p2, 64, 64))
    st = gpu_ctx.last_stats()
    assert st["error_flags"] == 0 and st["n_samples"] > 0
    v.close()
    tf.close()


@pytest.fixture(scope="module")
def flaky_plugin(native, tmp_path_factory):
    import shutil
    import livre_gb300 as lv
    from conftest import compile_against_include
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("flaky")
    compile_against_include(os.path.join(HERE, "plugins", "flaky_source.cpp"),
                            str(d / "libLivreFlakySource.so"), shared=True)
    assert lv.load_plugins(str(d)) == 1
    return d


def _frame(ctx, vol, tf, W=96, H=80):
    import livre_gb300 as lv
    mv, proj = lv.orbit_camera(2, 8, (1.0, 1.0, 1.0), W, H, radius_scale=1.2)
    img = ctx.render(vol, tf, ctx.render_desc(mv, proj, W, H, sse=1.0)).cpu().numpy()
    return img, ctx.last_stats()


@pytest.mark.parametrize("threads", [1, 4])
def test_plugin_getdata_throws_or_sleeps(gpu_ctx, flaky_plugin, threads):
    import time
    import livre_gb300 as lv
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf(256))
    gpu_ctx.purge()
    vol = gpu_ctx.open_volume("flaky://#192,32,30")
    vol.fetch_threads = threads
    t0 = time.perf_counter()
    img, st = _frame(gpu_ctx, vol, tf)
    elapsed = time.perf_counter() - t0
    resident = vol.resident()
    thrown = st["n_visible"] - st["n_uploaded"]
    assert thrown > 0 and st["n_uploaded"] > 0          # some skipped, the rest streamed
    assert all(lv.NodeId(r).position[0] != 1 for r in resident)
    slow = [r for r in resident if lv.NodeId(r).position[1] == 1]
    assert slow and elapsed >= 0.03                      # slow bricks arrived, late
    # the same volume through a callback that returns no data for those bricks
    info = vol.info

    def get_data(node_id, dst, nbytes):
        n = lv.NodeId(node_id)
        x, y, z = n.position
        if x == 1:
            return False
        C.memset(dst, 16 + (7 * x + 13 * y + 29 * z + 3 * n.level) % 200, nbytes)
        return True

    gpu_ctx.purge()
    ref_vol = gpu_ctx.callback_volume(info, get_data)
    ref, ref_st = _frame(gpu_ctx, ref_vol, tf)
    assert ref_st["n_uploaded"] == st["n_uploaded"]
    np.testing.assert_array_equal(img, ref)
    ref_vol.close()
    vol.close()
    tf.close()
