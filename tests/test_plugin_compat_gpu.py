"""A volume served by a data-source plugin (tests/plugins/checker_source.cpp,
registered through lunchbox::PluginRegisterer) rendered on the device and
checked against the oracle ray cast of the same bricks.

Tolerance: max per-channel |GPU - oracle| <= 1/255 (FP32 kernel, FP64 oracle).
"""
import numpy as np
import pytest

from test_plugin_compat import CHECKER, checker_brick

pytestmark = pytest.mark.gpu
TOL = 1.0 / 255.0


@pytest.mark.parametrize("bits", [8, 16])
def test_plugin_volume_renders_like_the_oracle(gpu_ctx, oracle, checker_plugin, bits):
    import livre_gb300 as lv
    uri = CHECKER + (",16" if bits == 16 else "")
    v = gpu_ctx.open_volume(uri)
    info = v.info
    dtype = 2 if bits == 16 else 1
    assert info.dtype == dtype and info.max_block == (34, 34, 34)
    # the pool is fed the plugin's bytes
    for nid in list(info.all_nodes())[:3]:
        np.testing.assert_array_equal(v.get_data(nid.id), checker_brick(info, nid))
    ovol = oracle.volume(info.voxels, 32, 1)
    tf_rgba = lv.linear_ramp_tf(256)
    tf = gpu_ctx.transfer_function(tf_rgba)
    W, H = 96, 80
    with lv.DataSource(uri) as src:
        for k in range(3):
            mv, proj = lv.orbit_camera(k, 8, info.world_size, W, H, radius_scale=1.2)
            img = gpu_ctx.render(v, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0,
                                                            step_policy=1)).cpu().numpy()
            st = gpu_ctx.last_stats()
            ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
            assert st["n_rendered"] == len(ids) > 0
            bricks = np.stack([src.get_data(int(i)) for i in ids])
            view = oracle.make_view(mv, proj, W, H, st["samples_per_ray"],
                                    range_hi=65535.0 if bits == 16 else 255.0)
            ref, ns = oracle.raycast(ovol, dtype, ids, bricks, tf_rgba, view)
            assert ns > 1000
            err = np.abs(img - ref).max()
            assert err <= TOL, (k, err)
    tf.close()
    v.close()
