"""Multi-pass frames: a visible set larger than the brick pool is rendered in
passes of at most a pool's worth of bricks, front to back by brick distance
(renderSync, RenderPipeline.cpp:92-158), each pass compositing on top of the
previous ones with the first pass's sampling rate. The oracle renders the
same passes with the FP64 per-ray caster (each pass starting from the image
of the previous ones): max channel error <= 1/255, and with early ray
termination off the composited-sample counts are equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1.0 / 255.0
PER_PASS = 64


def distance_order(ovol, ids, mv):
    """Brick order of DistanceOperator (RayCastRenderer.cpp:57-81): FP32
    distance of the LODNode box centre (DataSourcePlugin.cpp:40-71) in eye
    space, ties by node id."""
    f32 = np.float32
    m = np.asarray(mv, f32)  # column-major 4x4
    ws = [f32(ovol.world_size[a]) for a in range(3)]
    dist = []
    for i in ids:
        i = int(i)
        level = i & 0xF
        pos = [(i >> 4) & 0x3FFF, (i >> 18) & 0x3FFF, (i >> 32) & 0x3FFF]
        bricks = [int(ovol.root_blocks[a]) << level for a in range(3)]
        big = max(range(3), key=lambda a: (bricks[a], -a))
        denom = f32(bricks[big])
        c = []
        for a in range(3):
            half = ws[a] * f32(0.5)
            lo = f32(pos[a]) / denom * ws[a] - half
            hi = f32(pos[a] + 1) / denom * ws[a] - half
            c.append((lo + hi) * f32(0.5))
        e = [m[k] * c[0] + m[4 + k] * c[1] + m[8 + k] * c[2] + m[12 + k] for k in range(3)]
        dist.append(np.sqrt(f32(e[0] * e[0] + e[1] * e[1] + e[2] * e[2])))
    keys = sorted(range(len(ids)), key=lambda k: (float(dist[k]), int(ids[k])))
    return [int(ids[k]) for k in keys]


def oracle_passes(oracle, ovol, ids, mv, proj, W, H, n_samples, tf, early, seed):
    ordered = distance_order(ovol, ids, mv)
    bp = oracle.blob_params(12, seed, 0, 1)
    view = oracle.make_view(mv, proj, W, H, n_samples, early_exit=early)
    out, total = None, 0
    for p in range(0, len(ordered), PER_PASS):
        sub = ordered[p:p + PER_PASS]
        bricks = np.stack([oracle.blob_brick(ovol, bp, i) for i in sub])
        out, ns = oracle.raycast(ovol, 1, sub, bricks, tf, view, init=out)
        total += ns
    return out, total, ordered


@pytest.mark.parametrize("early,k", [(0.98, 1), (1.0, 5)])
def test_multipass_matches_oracle(oracle, early, k):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 16, 1)
    ovol = oracle.volume(128, 16, 1)
    ctx = lv.Context(0, pool_bytes=PER_PASS * vi.slot_bytes)
    try:
        vol = ctx.blob_volume(vi, 12, 7)
        tf_rgba = lv.gaussian_peaks_tf(256, seed=5)
        tf = ctx.transfer_function(tf_rgba)
        W, H = 96, 72
        mv, proj = lv.orbit_camera(k, 8, vi.world_size, W, H, radius_scale=1.05)
        desc = ctx.render_desc(mv, proj, W, H, sse=0.5, early_exit=early)
        img = ctx.render(vol, tf, desc).cpu().numpy()
        st = ctx.last_stats()
        ids, _ = oracle.select_visible(ovol, mv, proj, H, 0.5)
        assert st["n_visible"] == len(ids) > PER_PASS
        assert st["n_passes"] == (len(ids) + PER_PASS - 1) // PER_PASS
        assert st["n_not_available"] == 0 and st["error_flags"] == 0
        ref, ns, ordered = oracle_passes(oracle, ovol, ids, mv, proj, W, H,
                                         st["samples_per_ray"], tf_rgba, early, 7)
        # the sampling rate comes from the first pass's finest level
        top = max(lv.NodeId(i).level for i in ordered[:PER_PASS])
        assert st["samples_per_ray"] == (2 * 128) >> (vi.depth - 1 - top)
        assert np.abs(img - ref).max() <= TOL
        if early >= 1.0:
            assert st["n_samples"] == ns
        vol.close()
        tf.close()
    finally:
        ctx.close()


def test_one_pass_when_the_set_fits(oracle):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 16, 1)
    ctx = lv.Context(0, pool_bytes=PER_PASS * vi.slot_bytes)
    try:
        vol = ctx.blob_volume(vi, 12, 7)
        tf = ctx.transfer_function(lv.linear_ramp_tf())
        mv, proj = lv.orbit_camera(0, 8, vi.world_size, 64, 48, radius_scale=2.0)
        ctx.render(vol, tf, ctx.render_desc(mv, proj, 64, 48, sse=8.0))
        st = ctx.last_stats()
        assert st["n_visible"] <= PER_PASS and st["n_passes"] == 1
        vol.close()
        tf.close()
    finally:
        ctx.close()
