"""Ray-cast launch shapes: the tile-queue and warp-refill kernels take exactly
the samples of the one-thread-per-pixel kernel, in the same order, so every
launch kind and shape must give a bit-identical image and the same sample
count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAUNCHES = [(0, 8, 4, 0, 0, 0), (0, 16, 16, 0, 0, 1), (0, 32, 2, 0, 0, 0),
            (1, 8, 16, 0, 0, 1), (1, 16, 16, 0, 1, 0), (1, 8, 8, 0, 1, 1), (1, 32, 1, 0, 0, 0),
            (2, 8, 8, 8, 0, 0), (2, 8, 4, 1, 1, 0), (2, 16, 8, 2, 0, 0), (2, 16, 16, 32, 1, 0),
            (2, 32, 32, 64, 0, 0), (2, 32, 1, 5, 0, 0), (3, 8, 16, 0, 1, 0),
            (3, 8, 16, 0, 1, 1), (3, 16, 16, 0, 0, 1), (3, 32, 1, 0, 1, 0), (4, 8, 4, 0, 1, 1)]


def scenes(ctx, lv):
    """Volumes covering both voxel types, both filters and the clamped-edge
    variant (overlap 0), with viewports that are not tile multiples."""
    out = []
    specs = [(lv.VolumeInformation(128, 32, 1), 1, 0, (96, 80)),
             (lv.VolumeInformation(96, 16, 1, dtype=lv.DT_UINT16), 1, 3, (33, 57)),
             (lv.VolumeInformation((128, 96, 64), 16, 0), 0, 0, (70, 41)),
             (lv.VolumeInformation(64, 16, 0, dtype=lv.DT_UINT16), 1, 0, (5, 3)),
             # 32^3 / 64^3 / 128^3 bricks + overlap 1: the default launch's
             # fixed-pitch paths
             (lv.VolumeInformation(96, 32, 1, dtype=lv.DT_UINT16), 1, 1, (40, 24)),
             (lv.VolumeInformation(192, 64, 1), 1, 2, (64, 48)),
             (lv.VolumeInformation(256, 128, 1), 1, 0, (48, 40)),
             (lv.VolumeInformation((128, 192, 96), 64, 1, dtype=lv.DT_UINT16), 1, 0, (50, 70))]
    for k, (vi, filt, noise, (W, H)) in enumerate(specs):
        vol = ctx.blob_volume(vi, 9, 20 + k, noise)
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.1 + 0.2 * k)
        desc = ctx.render_desc(mv, proj, W, H, sse=1.0, filt=filt, early_exit=0.95)
        out.append((vol, desc))
    return out


def test_refill_launches_bit_identical(gpu_ctx):
    import torch
    import livre_gb300 as lv
    tf = gpu_ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=2))
    items = scenes(gpu_ctx, lv)
    default = gpu_ctx.render_launch()
    try:
        gpu_ctx.set_render_launch(lv.LAUNCH_GRID, 8, 16)  # one thread per pixel
        refs = []
        for vol, desc in items:
            refs.append((gpu_ctx.render(vol, tf, desc).clone(), gpu_ctx.last_stats()))
        for kind, tw, th, chk, order, la in LAUNCHES:
            gpu_ctx.set_render_launch(kind, tw, th, chk, order, la)
            for (vol, desc), (ref, rst) in zip(items, refs):
                img = gpu_ctx.render(vol, tf, desc)
                st = gpu_ctx.last_stats()
                assert torch.equal(img, ref), (kind, tw, th, chk, order, la, desc.width,
                                               desc.height)
                assert st["n_samples"] == rst["n_samples"]
                assert st["error_flags"] == 0
    finally:
        gpu_ctx.set_render_launch(**default)
    for vol, _ in items:
        vol.close()
    tf.close()


def test_render_launch_validation(gpu_ctx):
    import livre_gb300 as lv
    for bad in [(2, 4, 4, 8), (2, 64, 32, 8), (2, 8, 8, 0), (2, 8, 8, 65), (0, 8, 3, 0),
                (0, 32, 16, 0), (1, 4, 4, 0), (5, 8, 8, 8), (4, 8, 8, 0), (0, 8, 16, 0, 1),
                (1, 8, 16, 0, 2), (1, 8, 16, 0, 0, 2), (2, 8, 8, 8, 0, 1)]:
        with pytest.raises(lv.LivreError):
            gpu_ctx.set_render_launch(*bad)
    assert gpu_ctx.render_launch() == {"kind": 3, "tile_w": 8, "tile_h": 8,
                                       "samples_per_check": 0, "order": 1, "lookahead": 1}


@pytest.mark.parametrize("cfg", [
    dict(queue=1, tile_w=8, tile_h=8, samples_per_check=8),
    dict(queue=1, tile_w=16, tile_h=16, samples_per_check=1),
    dict(queue=1, tile_w=32, tile_h=4, samples_per_check=64, ctas_per_sm=2),
    dict(queue=0, tile_w=16, tile_h=8),
    dict(queue=0, tile_w=16, tile_h=8, order=0),
    dict(queue=0, tile_w=8, tile_h=8, tf_shared=1, ctas_per_sm=3),
    dict(queue=0, tile_w=8, tile_h=16, tf_shared=1, order=0),
    dict(queue=2, tile_w=8, tile_h=16),
    dict(queue=2, tile_w=8, tile_h=16, lookahead=1),
    dict(queue=2, tile_w=16, tile_h=16, order=0),
])
def test_batch_queue_kinds_match_single_views(gpu_ctx, cfg):
    """Both work-queue kinds, with and without graphs, give each view the
    image lv_render gives it alone."""
    import torch
    import livre_gb300 as lv
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())
    items = scenes(gpu_ctx, lv)
    singles = [gpu_ctx.render(v, tf, d).clone() for v, d in items]
    batch = lv.Batch(gpu_ctx)
    for use_graph in (1, 0):
        batch.set_config(use_graph=use_graph, **cfg)
        outs = [torch.zeros((d.height, d.width, 4), dtype=torch.float32, device="cuda")
                for _, d in items]
        for _ in range(2):
            batch.render([(v, tf, d, o) for (v, d), o in zip(items, outs)])
            stats = batch.stats(len(items))[0]
            assert all(s["error_flags"] == 0 for s in stats)
            for a, b in zip(singles, outs):
                assert torch.equal(a, b)
    batch.close()
    for vol, _ in items:
        vol.close()
    tf.close()


def test_padded_batches_share_graphs(gpu_ctx):
    """Batch sizes 5..8 run as one padded launch of 8 views: one capture,
    then replays, each size still matching lv_render."""
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1)
    vol = gpu_ctx.blob_volume(vi, 8, 5)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())
    views = []
    for k in range(8):
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, 40, 24, radius_scale=1.3)
        d = gpu_ctx.render_desc(mv, proj, 40, 24, sse=1.0)
        views.append((vol, tf, d, torch.zeros((24, 40, 4), dtype=torch.float32,
                                              device="cuda")))
    singles = [gpu_ctx.render(v, t, d).clone() for v, t, d, _ in views]
    batch = lv.Batch(gpu_ctx)
    batch.set_config(queue=lv.QUEUE_CTA_TILES, tile_w=8, tile_h=16)  # the graphed kind
    for n in (5, 6, 7, 8, 5):
        batch.render(views[:n])
        for (_, _, _, o), ref in zip(views[:n], singles):
            assert torch.equal(o, ref), n
    captures, replays, cached = batch.graph_stats()
    assert captures == 1 and replays == 4 and cached == 1
    batch.close()
    vol.close()
    tf.close()
