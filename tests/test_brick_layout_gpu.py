"""Brick layouts of the pool (lv_pool_set_brick_layout): uint8 bricks of 64
to 1024 voxels per row are stored as voxel quads by default (each voxel with
its +x, +y and +x+y neighbours; written canonical and expanded in place on
the device, or gathered from a page-locked host store straight into quads),
one voxel per byte with LV_BRICKS_COMPACT. The layout is internal: every
frame and histogram must be bit for bit the same in both, for every way a
brick reaches the pool (device generator, host store, a data-source
callback) and every ray-cast path (fixed-pitch look-ahead tiles, the generic
pitch of the other launch kinds, nearest filtering)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(ctx, lv, source, block=64):
    vi = lv.VolumeInformation(256, block, 1)  # (block + 2)^3 slots: quads by default
    if source == "device":
        return vi, ctx.blob_volume(vi, 24, 11, 4)
    if source == "host":
        return vi, ctx.blob_volume(vi, 24, 11, 4, placement=lv.BLOB_HOST)

    def get_data(node_id, dst, nbytes):
        brick = np.random.default_rng(node_id).integers(0, 256, nbytes, dtype=np.uint8)
        ctypes.memmove(dst, brick.ctypes.data, nbytes)
        return True
    return vi, ctx.callback_volume(vi, get_data)


@pytest.mark.parametrize("source,block", [("device", 64), ("host", 64), ("callback", 64),
                                          ("device", 128), ("host", 128)])
def test_quads_equal_compact(source, block):
    import livre_gb300 as lv
    frames = {}
    n = (block + 2) ** 3
    for layout in (lv.BRICKS_QUADS, lv.BRICKS_COMPACT):
        ctx = lv.Context(0, pool_bytes=512 << 20, brick_layout=layout)
        vi, vol = make(ctx, lv, source, block)
        assert ctx.slot_bytes(vi) == (((3 * n + 255) // 256 * 256 + n + 1023) // 1024 * 1024
                                      if layout == lv.BRICKS_QUADS else (n + 1023) // 1024 * 1024)
        tf = ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=9))
        out = []
        for k, (kind, filt, lookahead) in enumerate([
                (lv.LAUNCH_TILE_GRID, lv.FILTER_TRILINEAR, 1),   # pitch-66 kernel
                (lv.LAUNCH_GRID, lv.FILTER_TRILINEAR, 0),        # generic pitch
                (lv.LAUNCH_TILE_GRID, lv.FILTER_NEAREST, 1)]):   # one voxel per tap
            ctx.set_render_launch(kind, 8, 8, 0, lv.ORDER_LONGEST_FIRST if kind else
                                  lv.ORDER_RASTER, lookahead)
            mv, proj = lv.orbit_camera(3 + 5 * k, 16, vi.world_size, 160, 120,
                                       radius_scale=1.1)
            d = ctx.render_desc(mv, proj, 160, 120, sse=1.0, filt=filt, early_exit=0.995)
            img = ctx.render(vol, tf, d).cpu().numpy()
            st = ctx.last_stats()
            assert st["error_flags"] == 0 and st["n_not_available"] == 0
            out.append((img, st["n_samples"]))
        out.append((vol.histogram(vol.resident(), n_bins=64), 0))
        frames[layout] = out
        vol.close()
        tf.close()
        ctx.close()
    quads, compact = frames[lv.BRICKS_QUADS], frames[lv.BRICKS_COMPACT]
    for (a, na), (b, nb) in zip(quads[:-1], compact[:-1]):
        assert na == nb and na > 0
        assert np.array_equal(a, b)
    assert np.array_equal(quads[-1][0], compact[-1][0]) and quads[-1][0].sum() > 0


def test_layout_fixed_once_the_pool_exists():
    import livre_gb300 as lv
    from livre_gb300 import _abi
    ctx = lv.Context(0, pool_bytes=64 << 20)
    vol = ctx.blob_volume(lv.VolumeInformation(128, 64, 1), 4, 1)  # allocates the pool
    assert _abi.lib().lv_pool_set_brick_layout(ctx.handle, lv.BRICKS_COMPACT) == _abi.LV_EINVAL
    assert _abi.lib().lv_pool_set_brick_layout(ctx.handle, 7) == _abi.LV_EINVAL
    vol.close()
    ctx.close()
