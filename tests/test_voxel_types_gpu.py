"""Ray casting volumes of every voxel type the reference's shader takes
(RayCastRenderer.cpp:236-277: unsigned, signed and float textures), against
the oracle. The int8 / int16 / uint32 / int32 / float volumes hold the blob
volume's uint8 bricks under an affine map; with the data range mapped the
same way, each renders like the uint8 volume.

Tolerance: max per-channel |GPU - oracle| <= 1/255.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1.0 / 255.0

# lv_dtype, numpy type, value map of a uint8 voxel v, data range (None: the
# type's own range)
TYPES = [
    (4, np.int8, lambda v: v.astype(np.int16) - 128, None),
    (5, np.int16, lambda v: v.astype(np.int32) * 100 - 12000, (-12000.0, 13500.0)),
    (3, np.uint32, lambda v: v.astype(np.uint64) * 16777, (0.0, 255.0 * 16777)),
    (6, np.int32, lambda v: v.astype(np.int64) * 1000 - 100000, (-100000.0, 155000.0)),
    (0, np.float32, lambda v: v.astype(np.float64) / 255.0 * 3.5 - 1.0, (-1.0, 2.5)),
]


def typed_volume(ctx, oracle, lv, dtype, ntype, vmap):
    vi = lv.VolumeInformation(128, 32, 1, dtype=dtype)
    ovol = oracle.volume(128, 32, 1)
    bp = oracle.blob_params(10, 7, 0, 1)
    bricks = {}
    for nid in vi.all_nodes():
        b8 = oracle.blob_brick(ovol, bp, nid.id)
        bricks[nid.id] = np.ascontiguousarray(vmap(b8).astype(ntype))

    def get_data(node_id, dst, nbytes):
        b = bricks.get(node_id)
        if b is None or b.nbytes != nbytes:
            return False
        C.memmove(dst, b.ctypes.data, nbytes)
        return True

    return vi, ovol, ctx.callback_volume(vi, get_data), bricks


@pytest.mark.parametrize("dtype,ntype,vmap,rng", TYPES)
@pytest.mark.parametrize("filt", [0, 1])
def test_voxel_type_renders_like_the_oracle(gpu_ctx, oracle, dtype, ntype, vmap, rng, filt):
    import livre_gb300 as lv
    vi, ovol, vol, bricks = typed_volume(gpu_ctx, oracle, lv, dtype, ntype, vmap)
    tf_rgba = lv.linear_ramp_tf(256)
    tf = gpu_ctx.transfer_function(tf_rgba)
    W, H = 80, 64
    for k in (1, 4):
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.2)
        desc = gpu_ctx.render_desc(mv, proj, W, H, sse=1.0, filt=filt,
                                   data_range=rng or (0.0, 0.0))
        img = gpu_ctx.render(vol, tf, desc).cpu().numpy()
        st = gpu_ctx.last_stats()
        assert st["error_flags"] == 0
        ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
        assert st["n_rendered"] == len(ids) > 0
        lo, hi = rng or (-128.0, 127.0)
        view = oracle.make_view(mv, proj, W, H, st["samples_per_ray"], filt=filt,
                                range_lo=lo, range_hi=hi)
        stack = np.stack([bricks[int(i)] for i in ids])
        ref, ns = oracle.raycast(ovol, dtype, ids, stack, tf_rgba, view)
        assert ns > 500
        err = np.abs(img - ref).max()
        assert err <= TOL, (k, err)
    vol.close()
    tf.close()


def test_float_volume_type_range_maps_to_the_first_entry(gpu_ctx, oracle):
    """With no data range a float volume uses [FLT_MIN, FLT_MAX], as the
    reference does, so every sample reads the transfer function's first
    entry."""
    import livre_gb300 as lv
    vi, ovol, vol, bricks = typed_volume(gpu_ctx, oracle, lv, 0, np.float32,
                                         lambda v: v.astype(np.float64) / 255.0)
    tf_rgba = lv.linear_ramp_tf(256)
    tf_rgba[0] = (0.2, 0.4, 0.6, 0.05)
    tf = gpu_ctx.transfer_function(tf_rgba)
    mv, proj = lv.orbit_camera(2, 8, vi.world_size, 48, 40, radius_scale=1.2)
    img = gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, 48, 40, sse=1.0)).cpu().numpy()
    st = gpu_ctx.last_stats()
    ids, _ = oracle.select_visible(ovol, mv, proj, 40, 1.0)
    view = oracle.make_view(mv, proj, 48, 40, st["samples_per_ray"],
                            range_lo=1.17549435e-38, range_hi=3.40282347e38)
    ref, _ = oracle.raycast(ovol, 0, ids, np.stack([bricks[int(i)] for i in ids]), tf_rgba,
                            view)
    assert np.abs(img - ref).max() <= TOL
    covered = img[..., 3] > 0
    assert covered.any()
    rgb = img[..., :3][covered] / img[..., 3][covered][:, None]
    np.testing.assert_allclose(rgb, np.broadcast_to([0.2, 0.4, 0.6], rgb.shape), atol=1e-4)
    vol.close()
    tf.close()


def test_batches_of_other_voxel_types(gpu_ctx, oracle):
    """View kernels render any voxel type and match lv_render; the persistent
    queues refuse them."""
    import torch
    import livre_gb300 as lv
    dtype, ntype, vmap, rng = TYPES[1]
    vi, ovol, vol, _ = typed_volume(gpu_ctx, oracle, lv, dtype, ntype, vmap)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf(256))
    views = []
    for k in range(3):
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, 40, 32, radius_scale=1.3)
        d = gpu_ctx.render_desc(mv, proj, 40, 32, sse=1.0, data_range=rng)
        views.append((vol, tf, d, torch.zeros((32, 40, 4), dtype=torch.float32,
                                              device="cuda")))
    singles = [gpu_ctx.render(v, t, d).clone() for v, t, d, _ in views]
    batch = lv.Batch(gpu_ctx)
    batch.set_config(queue=lv.QUEUE_VIEW_KERNELS)
    batch.render(views)
    for (_, _, _, o), ref in zip(views, singles):
        assert torch.equal(o, ref)
    batch.set_config(queue=lv.QUEUE_CTA_TILES)
    with pytest.raises(lv.LivreError):
        batch.render(views)
    batch.close()
    vol.close()
    tf.close()


@pytest.mark.parametrize("dtype,ntype,vmap,rng", TYPES)
def test_histograms_of_other_voxel_types(gpu_ctx, oracle, dtype, ntype, vmap, rng):
    """lv_histogram bins every voxel type with the same rule as uint8/uint16:
    floor((v - lo) * (n - 1) / (hi - lo)) clamped, counts weighted by the
    finest voxels one voxel stands for, the overlap skipped."""
    import livre_gb300 as lv
    vi, ovol, vol, bricks = typed_volume(gpu_ctx, oracle, lv, dtype, ntype, vmap)
    lo, hi = rng or (-128.0, 127.0)
    n_bins = 100
    ids = [lv.NodeId(0, (0, 0, 0)).id, lv.NodeId(1, (1, 0, 1)).id, lv.NodeId(2, (3, 2, 0)).id]
    acc, per = vol.histogram(ids, n_bins, (lo, hi), per_brick=True)
    scale_bins = np.float32(n_bins - 1) / (np.float32(hi) - np.float32(lo))
    want_acc = np.zeros(n_bins, np.uint64)
    for k, i in enumerate(ids):
        b = bricks[i].reshape(34, 34, 34)[1:33, 1:33, 1:33].astype(np.float32)
        f = np.floor((b - np.float32(lo)) * np.float32(scale_bins))
        bins = np.clip(f, 0, n_bins - 1).astype(np.int64)
        scale = (2 ** (vi.depth - 1 - (i & 0xF))) ** 3
        h = np.bincount(bins.ravel(), minlength=n_bins).astype(np.uint64) * np.uint64(scale)
        assert (per[k] == h).all(), k
        want_acc += h
    assert (acc == want_acc).all()
    vol.close()
