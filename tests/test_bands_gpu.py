"""Sort-first bands (lv_render_desc.rect): a frame rendered as bands of rows
and stitched equals the frame rendered whole, bit for bit, for every launch
kind and in batches; pixels outside a rect are not written."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAUNCHES = [(3, 8, 16, 0, 1, 1), (3, 8, 16, 0, 1, 0), (0, 8, 16, 0, 0, 0), (1, 16, 8, 0, 1, 0),
            (2, 8, 8, 8, 0, 0), (4, 8, 4, 0, 1, 1)]


def scene(ctx, lv, dtype=1):
    vi = lv.VolumeInformation(128, 32, 1, dtype=dtype)
    vol = ctx.blob_volume(vi, 9, 4, 2)
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=3))
    mv, proj = lv.orbit_camera(3, 8, vi.world_size, 77, 53, radius_scale=1.2)
    return vi, vol, tf, mv, proj


@pytest.mark.parametrize("launch", LAUNCHES)
def test_bands_stitch_to_the_whole_frame(gpu_ctx, launch):
    import torch
    import livre_gb300 as lv
    from livre_gb300 import replicas
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv)
    W, H = 77, 53
    default = gpu_ctx.render_launch()
    try:
        gpu_ctx.set_render_launch(*launch)
        full = gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0)).clone()
        n_full = gpu_ctx.last_stats()["n_samples"]
        for world in (2, 3, 5):
            out = torch.full((H, W, 4), -7.0, device="cuda")
            n = 0
            for r in range(world):
                y0, rows = replicas.band(H, r, world)
                d = gpu_ctx.render_desc(mv, proj, W, H, sse=1.0, rect=(0, y0, W, rows))
                gpu_ctx.render(vol, tf, d, out)
                n += gpu_ctx.last_stats()["n_samples"]
            assert torch.equal(out, full), world
            assert n == n_full
    finally:
        gpu_ctx.set_render_launch(**default)
    vol.close()
    tf.close()


def test_rect_writes_only_its_pixels(gpu_ctx):
    import torch
    import livre_gb300 as lv
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv, dtype=2)
    W, H = 77, 53
    full = gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0)).clone()
    out = torch.full((H, W, 4), -7.0, device="cuda")
    x, y, w, h = 9, 11, 40, 23
    gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0, rect=(x, y, w, h)), out)
    inside = torch.zeros((H, W), dtype=torch.bool, device="cuda")
    inside[y:y + h, x:x + w] = True
    assert torch.equal(out[inside], full[inside])
    assert bool((out[~inside] == -7.0).all())
    for bad in [(70, 0, 8, 10), (0, 50, 10, 4), (0xFFFFFFF0, 0, 32, 1)]:
        with pytest.raises(lv.LivreError):
            gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, rect=bad), out)
    vol.close()
    tf.close()


@pytest.mark.parametrize("queue", [0, 2])
def test_batched_bands(gpu_ctx, queue):
    """A batch of the bands of two frames fills both frames."""
    import torch
    import livre_gb300 as lv
    from livre_gb300 import replicas
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv)
    W, H = 77, 53
    mv2, proj2 = lv.orbit_camera(6, 8, vi.world_size, W, H, radius_scale=1.4)
    fulls = [gpu_ctx.render(vol, tf, gpu_ctx.render_desc(m, p, W, H, sse=1.0)).clone()
             for m, p in ((mv, proj), (mv2, proj2))]
    outs = [torch.full((H, W, 4), -7.0, device="cuda") for _ in range(2)]
    items = []
    for (m, p), o in zip(((mv, proj), (mv2, proj2)), outs):
        for r in range(3):
            y0, rows = replicas.band(H, r, 3)
            items.append((vol, tf, gpu_ctx.render_desc(m, p, W, H, sse=1.0,
                                                         rect=(0, y0, W, rows)), o))
    batch = lv.Batch(gpu_ctx)
    batch.set_config(queue=queue)
    batch.render(items)
    torch.cuda.synchronize()
    for o, f in zip(outs, fulls):
        assert torch.equal(o, f)
    batch.close()
    vol.close()
    tf.close()


def test_band_histograms_add_up_to_the_frame(gpu_ctx, oracle):
    """HistogramFilter's per-view histogram: every brick of the frame counts
    once over the whole frame, and the bands' histograms add up to it."""
    import numpy as np
    import livre_gb300 as lv
    from livre_gb300 import replicas
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv)
    W, H = 77, 53
    gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0))
    whole = gpu_ctx.frame_histogram(64, (0.0, 255.0))
    ovol = oracle.volume(128, 32, 1)
    ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
    np.testing.assert_array_equal(whole, vol.histogram([int(i) for i in ids], 64, (0.0, 255.0)))
    for world in (2, 3, 4):
        total = np.zeros(64, np.uint64)
        nonempty = 0
        for r in range(world):
            y0, rows = replicas.band(H, r, world)
            gpu_ctx.render(vol, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0,
                                                         rect=(0, y0, W, rows)))
            part = gpu_ctx.frame_histogram(64, (0.0, 255.0))
            nonempty += int(part.sum() > 0)
            total += part
        np.testing.assert_array_equal(total, whole)
        assert nonempty >= 2  # the bricks split between bands
    vol.close()
    tf.close()


def test_frames_on_different_streams_stay_ordered(gpu_ctx):
    """lv_render returns with its ray cast queued; consecutive frames on
    different streams reuse the same per-frame buffers and must not overlap.
    Each frame, rendered back to back on alternating streams with no host
    wait, equals the same frame rendered alone."""
    import torch
    import livre_gb300 as lv
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv)
    W, H = 77, 53
    cams = [lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.1 + 0.1 * k)
            for k in range(6)]
    descs = [gpu_ctx.render_desc(m, p, W, H, sse=1.0) for m, p in cams]
    alone = []
    for d in descs:
        alone.append(gpu_ctx.render(vol, tf, d).clone())
        torch.cuda.synchronize()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    outs = [torch.empty((H, W, 4), dtype=torch.float32, device="cuda") for _ in descs]
    for k, (d, o) in enumerate(zip(descs, outs)):
        gpu_ctx.render(vol, tf, d, o, stream=streams[k % 2])
    torch.cuda.synchronize()
    for o, a in zip(outs, alone):
        assert torch.equal(o, a)
    vol.close()
    tf.close()


def test_selections_between_queued_frames(gpu_ctx):
    """lv_render's selection and lv_select_visible share the context's
    frontier queues and run on different streams; frames queued back to back
    with selections of another view issued between them (on a third stream,
    no host wait) give the frames and visible sets each gives alone."""
    import torch
    import livre_gb300 as lv
    vi, vol, tf, mv, proj = scene(gpu_ctx, lv)
    W, H = 77, 53
    cams = [lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.1 + 0.1 * k)
            for k in range(6)]
    descs = [gpu_ctx.render_desc(m, p, W, H, sse=1.0) for m, p in cams]
    alone = [gpu_ctx.render(vol, tf, d).clone() for d in descs]
    sel_cams = [lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=2.0) for k in (1, 4)]
    sel_alone = [sorted(gpu_ctx.select_visible(vi, m, p, H, 0.5)[0].tolist()) for m, p in sel_cams]
    torch.cuda.synchronize()
    other = torch.cuda.Stream()
    outs = [torch.empty((H, W, 4), dtype=torch.float32, device="cuda") for _ in descs]
    # the selections' buffers, made before any frame is queued (a buffer
    # zeroed on the rendering stream would be zeroed after the frames)
    bufs = [(torch.empty(vi.node_count(), dtype=torch.int64, device="cuda"),
             torch.zeros(lv._abi.SELECT_RESULT_WORDS, dtype=torch.int32, device="cuda"))
            for _ in descs]
    torch.cuda.synchronize()
    pending = []
    for k, (d, o) in enumerate(zip(descs, outs)):
        gpu_ctx.render(vol, tf, d, o)
        m, p = sel_cams[k % 2]
        ids, res = bufs[k]
        pending.append((k % 2, gpu_ctx.select_visible(vi, m, p, H, 0.5, out=ids, result=res,
                                                      stream=other, sync=False)))
    torch.cuda.synchronize()
    for o, a in zip(outs, alone):
        assert torch.equal(o, a)
    for j, (ids, res) in pending:
        n = int(res.cpu().numpy().view("uint32")[lv._abi.SEL_WRITTEN])
        got = sorted(ids[:n].cpu().numpy().view("uint64").tolist())
        assert got == sel_alone[j]
    vol.close()
    tf.close()
