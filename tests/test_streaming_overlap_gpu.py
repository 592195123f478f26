"""Frames rendered back to back while bricks stream: a synchronous frame
queued while the previous one still ray casts looks its visible bricks up
beside that ray cast and streams the missing ones then, sparing every brick
the running frame reads. Each frame must equal the same frame rendered with
the host waiting between frames, bit for bit, through a pool that holds more
than a frame's bricks but not the whole fly-through's (so bricks are evicted
while earlier frames still render)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fly(lv, k, n, W, H):
    a, b = np.array([-0.45, -0.3, -0.8]), np.array([0.35, 0.25, 0.55])
    eye = a + (b - a) * (k / (n - 1))
    mv = lv.look_at(eye, eye + (b - a) / np.linalg.norm(b - a), (0.0, 1.0, 0.0))
    return mv, lv.perspective(45.0, W / H, 0.01, 15.0)


def make_volume(ctx, lv, placement):
    if placement == "callback":
        # a data-source callback (getData): bricks through the staging ring
        import ctypes
        vi = lv.VolumeInformation(512, 32, 1)

        def get_data(node_id, dst, nbytes):
            brick = np.random.default_rng(node_id).integers(0, 256, nbytes, dtype=np.uint8)
            ctypes.memmove(dst, brick.ctypes.data, nbytes)
            return True
        return vi, ctx.callback_volume(vi, get_data)
    if placement == "blob_host":
        vi = lv.VolumeInformation(512, 32, 1)
        return vi, ctx.blob_volume(vi, 48, 5, 4, placement=lv.BLOB_HOST)
    vi = lv.VolumeInformation(512, 32, 1, dtype=lv.DT_UINT16)
    return vi, ctx.fbm_volume(vi, 3, octaves=3, frequency=4.0, placement=lv.FBM_DEVICE)


@pytest.mark.parametrize("placement,pool", [("blob_host", "half"), ("fbm_device", "half"),
                                            ("blob_host", "tight"), ("fbm_device", "tight"),
                                            ("callback", "half"), ("callback", "tight")])
def test_back_to_back_frames_equal_waited_frames(native, placement, pool):
    import torch
    import livre_gb300 as lv
    W, H, n, path = 480, 320, 14, 24
    # reference: the host waits for every frame; a pool holding everything
    ctx = lv.Context(0, pool_bytes=1 << 30)
    vi, vol = make_volume(ctx, lv, placement)
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=6))
    descs = [ctx.render_desc(*fly(lv, k, path, W, H), W, H, sse=1.5, early_exit=0.999)
             for k in range(n)]
    waited, most = [], 0
    for d in descs:
        waited.append(ctx.render(vol, tf, d).clone())
        st = ctx.last_stats()
        assert st["error_flags"] == 0 and st["n_passes"] == 1
        most = max(most, st["n_visible"])
    union = ctx.totals()["bricks_uploaded"]
    slot = vi.slot_bytes
    vol.close()
    tf.close()
    ctx.close()
    # back to back through a pool halfway between one frame's bricks and the
    # whole fly-through's (consecutive frames share most of their bricks), or
    # through one frame's bricks and a slot: then a frame's misses cannot all
    # be placed beside the previous frame, whose bricks are all in use
    bricks = (most + union) // 2 if pool == "half" else most + 1
    print(placement, pool, "largest visible set", most, "distinct bricks", union, "pool", bricks)
    assert most < bricks < union, "the fly-through must outgrow the pool"
    ctx = lv.Context(0, pool_bytes=bricks * slot)
    vi, vol = make_volume(ctx, lv, placement)
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=6))
    outs = [torch.empty((H, W, 4), dtype=torch.float32, device="cuda") for _ in descs]
    for d, o in zip(descs, outs):
        ctx.render(vol, tf, d, o)  # no wait between frames
    st = ctx.last_stats()
    assert st["error_flags"] == 0
    torch.cuda.synchronize()
    assert ctx.totals()["bricks_uploaded"] > bricks  # evictions happened
    for k, (o, w) in enumerate(zip(outs, waited)):
        assert torch.equal(o, w), k
    vol.close()
    tf.close()
    ctx.close()
