"""Batched rendering (lv_batch_*): many views of several volumes in one
persistent launch replayed as a CUDA graph. Each view must equal the same view
rendered alone by lv_render, and the oracle within 1/255."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_views(ctx, lv, n=6, seed=0):
    rng = np.random.default_rng(seed)
    vols = [
        (lv.VolumeInformation(128, 32, 1), 12, 3, 0),
        (lv.VolumeInformation(96, 16, 1, dtype=lv.DT_UINT16), 9, 5, 2),
        (lv.VolumeInformation((128, 96, 64), 16, 1), 7, 8, 4),
    ]
    volumes = [(ctx.blob_volume(vi, nb, sd, noise), vi) for vi, nb, sd, noise in vols]
    tfs = [ctx.transfer_function(lv.linear_ramp_tf(256)),
           ctx.transfer_function(lv.gaussian_peaks_tf(1024, seed=3)),
           ctx.transfer_function(lv.default_transfer_function())]
    items = []
    sizes = [(64, 48), (40, 40), (96, 32), (33, 57), (80, 64), (16, 16)]
    for k in range(n):
        vol, vi = volumes[k % len(volumes)]
        W, H = sizes[k % len(sizes)]
        mv, proj = lv.orbit_camera(int(rng.integers(0, 16)), 16, vi.world_size, W, H,
                                   radius_scale=float(rng.uniform(0.9, 1.6)))
        desc = ctx.render_desc(mv, proj, W, H, sse=float(rng.uniform(0.5, 4.0)),
                               filt=int(k % 2 == 0), early_exit=0.999, synchronous=True)
        items.append((vol, tfs[k % len(tfs)], desc))
    return volumes, tfs, items


def test_batch_equals_single_views(gpu_ctx):
    import torch
    import livre_gb300 as lv
    volumes, tfs, items = make_views(gpu_ctx, lv)
    singles = []
    for vol, tf, desc in items:  # plain path, synchronous: loads every brick
        singles.append(gpu_ctx.render(vol, tf, desc).clone())
    batch = lv.Batch(gpu_ctx)
    outs = [torch.zeros((d.height, d.width, 4), dtype=torch.float32, device="cuda")
            for _, _, d in items]
    for rep in range(3):  # graph capture, then replays
        batch.render([(v, t, d, o) for (v, t, d), o in zip(items, outs)])
        stats, sel_ms, ray_ms = batch.stats(len(items))
        for i, (a, b) in enumerate(zip(singles, outs)):
            assert torch.equal(a, b) or float((a - b).abs().max()) <= 1e-6, (rep, i)
        assert all(s["n_not_available"] == 0 for s in stats)
        assert ray_ms > 0
    # the default queue (per-view kernels) runs each batch as one graph
    # launch: instantiated once, then the later captures update it
    caps, reps, cached = batch.graph_stats()
    assert batch.config()["queue"] == lv.QUEUE_VIEW_KERNELS
    assert (caps, reps) == (1, 2), (caps, reps)
    batch.close()
    for v, _ in volumes:
        v.close()
    for t in tfs:
        t.close()


def test_batch_matches_oracle(gpu_ctx, oracle):
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1)
    ovol = oracle.volume(128, 32, 1)
    vol = gpu_ctx.blob_volume(vi, 10, 6)
    tf_rgba = lv.gaussian_peaks_tf(256, seed=1)
    tf = gpu_ctx.transfer_function(tf_rgba)
    mv, proj = lv.orbit_camera(2, 8, vi.world_size, 72, 40, radius_scale=1.2)
    desc = gpu_ctx.render_desc(mv, proj, 72, 40, sse=1.0)
    ids, _ = oracle.select_visible(ovol, mv, proj, 40, 1.0)
    vol.load([int(i) for i in ids])
    batch = lv.Batch(gpu_ctx)
    out = torch.zeros((40, 72, 4), dtype=torch.float32, device="cuda")
    batch.render([(vol, tf, desc, out)])
    st = batch.stats(1)[0][0]
    bp = oracle.blob_params(10, 6, 0, 1)
    bricks = np.stack([oracle.blob_brick(ovol, bp, int(i)) for i in ids])
    ref, ns = oracle.raycast(ovol, 1, ids, bricks, tf_rgba,
                             oracle.make_view(mv, proj, 72, 40, st["samples_per_ray"]))
    assert np.abs(out.cpu().numpy() - ref).max() <= 1.0 / 255.0
    batch.close()
    vol.close()
    tf.close()


def test_batch_async_streams_misses(gpu_ctx):
    """A cold batch renders ancestors and converges to the full-resolution image."""
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1)
    vol = gpu_ctx.blob_volume(vi, 10, 9)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())
    mv, proj = lv.orbit_camera(4, 8, vi.world_size, 48, 48, radius_scale=1.1)
    desc = gpu_ctx.render_desc(mv, proj, 48, 48, sse=1.0, max_uploads=8)
    batch = lv.Batch(gpu_ctx)
    out = torch.zeros((48, 48, 4), dtype=torch.float32, device="cuda")
    done = False
    for _ in range(64):
        batch.render([(vol, tf, desc, out)])
        st = batch.stats(1)[0][0]
        if st["n_not_available"] == 0:
            done = True
            break
    assert done
    ref = gpu_ctx.render(vol, tf, desc)
    assert float((ref - out).abs().max()) <= 1e-6
    batch.close()
    vol.close()
    tf.close()


def test_autotune_picks_valid_config(gpu_ctx):
    import torch
    import livre_gb300 as lv
    volumes, tfs, items = make_views(gpu_ctx, lv, n=4, seed=1)
    for vol, tf, desc in items:
        gpu_ctx.render(vol, tf, desc)
    batch = lv.Batch(gpu_ctx)
    outs = [torch.zeros((d.height, d.width, 4), dtype=torch.float32, device="cuda")
            for _, _, d in items]
    packed = [(v, t, d, o) for (v, t, d), o in zip(items, outs)]
    cfg = batch.autotune(packed, reps=1)
    assert cfg["tile_w"] * cfg["tile_h"] in (32, 64, 128, 256)
    assert batch.config() == cfg
    batch.render(packed)
    singles = [gpu_ctx.render(v, t, d) for v, t, d in items]
    for a, b in zip(singles, outs):
        assert float((a - b).abs().max()) <= 1e-6
    batch.close()
    for v, _ in volumes:
        v.close()
    for t in tfs:
        t.close()


def test_graph_replay_with_new_composition(gpu_ctx):
    """The same batch object replays its captured graph for a new set of views
    with the same count and kernel variants but a different split between
    them and a different number of octree roots: every view still matches."""
    import torch
    import livre_gb300 as lv
    a = lv.VolumeInformation(128, 32, 1)
    b16 = lv.VolumeInformation(96, 16, 1, dtype=lv.DT_UINT16)
    c = lv.VolumeInformation((128, 96, 64), 16, 1)  # several root blocks
    va, vb, vc = (gpu_ctx.blob_volume(vi, 8, 40 + k) for k, vi in enumerate((a, b16, c)))
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())

    def view(vol, vi, k, W=40, H=32):
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.3)
        d = gpu_ctx.render_desc(mv, proj, W, H, sse=1.0)
        gpu_ctx.render(vol, tf, d)  # bricks resident
        return (vol, tf, d, torch.zeros((H, W, 4), dtype=torch.float32, device="cuda"))

    batch = lv.Batch(gpu_ctx)
    first = [view(va, a, 0), view(va, a, 1), view(vb, b16, 2)]
    second = [view(vc, c, 3), view(vb, b16, 4), view(vb, b16, 5)]  # 1 u8 + 2 u16, more roots
    for items in (first, second, first, second):
        batch.render(items)
        stats = batch.stats(len(items))[0]
        assert all(s["error_flags"] == 0 for s in stats)
        for v, t, d, o in items:
            ref = gpu_ctx.render(v, t, d)
            assert float((ref - o).abs().max()) <= 1e-6
    batch.close()
    for v in (va, vb, vc):
        v.close()
    tf.close()


def test_graph_cache_after_frontier_growth(gpu_ctx):
    """Batches of growing size reallocate the batch's frontier queues several
    times; replaying a smaller batch afterwards must use the new queues (the
    graph captured before the growth is dropped) and still match."""
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(256, 32, 1)
    vol = gpu_ctx.blob_volume(vi, 10, 77)
    tf = gpu_ctx.transfer_function(lv.linear_ramp_tf())
    views = []
    for k in range(12):
        mv, proj = lv.orbit_camera(k, 12, vi.world_size, 24, 24, radius_scale=1.2)
        d = gpu_ctx.render_desc(mv, proj, 24, 24, sse=1.0)
        gpu_ctx.render(vol, tf, d)
        views.append((vol, tf, d, torch.zeros((24, 24, 4), dtype=torch.float32, device="cuda")))
    batch = lv.Batch(gpu_ctx)
    for n in list(range(1, 13)) + [1, 3, 12, 2]:
        items = views[:n]
        batch.render(items)
        stats = batch.stats(n)[0]
        assert all(s["error_flags"] == 0 for s in stats)
        for v, t, d, o in items:
            assert float((gpu_ctx.render(v, t, d) - o).abs().max()) <= 1e-6, n
    batch.close()
    vol.close()
    tf.close()
