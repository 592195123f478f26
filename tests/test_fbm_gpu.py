"""fBm volumes on the device: the device generator gives the host
generator's bytes, host-generated (data-source callback) and device-generated
volumes render the same image, and the image matches the oracle within
1/255."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_fbm_matches_host(gpu_ctx):
    import livre_gb300 as lv
    for dt in (lv.DT_UINT16, lv.DT_UINT8):
        vi = lv.VolumeInformation((160, 96, 128), 32, 1, dtype=dt)
        ids = [n.id for n in vi.all_nodes()]
        dev = gpu_ctx.fbm_bricks(vi, ids, 77).cpu().numpy()
        for k, i in enumerate(ids):
            assert np.array_equal(dev[k], lv.fbm_brick(vi, i, 77, n_threads=8)), hex(i)


def test_fbm_volume_renders_like_oracle(gpu_ctx, oracle):
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1, dtype=lv.DT_UINT16)
    ovol = oracle.volume(128, 32, 1)
    tf_rgba = lv.gaussian_peaks_tf(1024, seed=8)
    tf = gpu_ctx.transfer_function(tf_rgba)
    vd = gpu_ctx.fbm_volume(vi, 31, frequency=4.0, placement=lv.FBM_DEVICE)
    vh = gpu_ctx.fbm_volume(vi, 31, frequency=4.0, placement=lv.FBM_HOST, host_threads=4)
    W, H = 80, 64
    mv, proj = lv.orbit_camera(3, 8, vi.world_size, W, H, radius_scale=1.1)
    desc = gpu_ctx.render_desc(mv, proj, W, H, sse=1.0, early_exit=0.99)
    a = gpu_ctx.render(vd, tf, desc).clone()
    st = gpu_ctx.last_stats()
    b = gpu_ctx.render(vh, tf, desc)
    assert torch.equal(a, b)
    ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
    fp = oracle.fbm_params(31, 6, 2.0, 0.5, 4.0, dtype=2)
    bricks = np.stack([oracle.fbm_brick(ovol, fp, int(i)) for i in ids])
    view = oracle.make_view(mv, proj, W, H, st["samples_per_ray"], early_exit=0.99,
                            range_lo=0.0, range_hi=65535.0)
    ref, _ = oracle.raycast(ovol, 2, ids, bricks, tf_rgba, view)
    assert np.abs(a.cpu().numpy() - ref).max() <= 1.0 / 255.0
    for v in (vd, vh):
        v.close()
    tf.close()
