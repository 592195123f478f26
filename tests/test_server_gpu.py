"""Render server (lv_server_*): continuous batching with admission by brick-pool
memory. Every request's frame must equal the same request rendered alone with
lv_render, whatever else was in its batch (tolerance 1e-6, in practice equal)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scene(ctx, lv, seed=0, n=12):
    rng = np.random.default_rng(seed)
    infos = [lv.VolumeInformation(128, 32, 1), lv.VolumeInformation(96, 16, 1, dtype=lv.DT_UINT16),
             lv.VolumeInformation(64, 16, 1)]
    vols = [ctx.blob_volume(vi, 8 + 3 * i, 20 + i, noise=i) for i, vi in enumerate(infos)]
    tfs = [ctx.transfer_function(lv.linear_ramp_tf(256)),
           ctx.transfer_function(lv.gaussian_peaks_tf(512, seed=5))]
    reqs = []
    for k in range(n):
        i = int(rng.integers(0, len(vols)))
        W, H = [(48, 32), (64, 64), (30, 70), (96, 54)][k % 4]
        mv, proj = lv.orbit_camera(int(rng.integers(0, 32)), 32, infos[i].world_size, W, H,
                                   radius_scale=float(rng.uniform(0.9, 1.8)))
        desc = ctx.render_desc(mv, proj, W, H, sse=float(rng.uniform(0.5, 4.0)),
                               filt=int(rng.integers(0, 2)))
        reqs.append((vols[i], tfs[k % 2], desc))
    return vols, tfs, reqs


def alone(ctx, reqs):
    outs = []
    for v, t, d in reqs:
        outs.append(ctx.render(v, t, d).clone())
    return outs


@pytest.mark.parametrize("mode", [0, 1])
def test_server_results_equal_alone(mode):
    import torch
    import livre_gb300 as lv
    ctx = lv.Context(0, pool_bytes=512 << 20)
    vols, tfs, reqs = scene(ctx, lv)
    srv = lv.Server(ctx, mode=mode, max_batch=8)
    outs = [torch.zeros((d.height, d.width, 4), dtype=torch.float32, device="cuda")
            for _, _, d in reqs]
    tickets = [srv.submit(v, t, d, o) for (v, t, d), o in zip(reqs, outs)]
    results = [srv.wait(tk) for tk in tickets]
    assert all(r["status"] == 0 for r in results)
    assert all(r["latency_ms"] >= r["queue_ms"] >= 0 for r in results)
    if mode == 0:
        assert max(r["batch_size"] for r in results) > 1
    srv.close()
    ref = alone(ctx, reqs)
    for i, (a, b) in enumerate(zip(ref, outs)):
        assert float((a - b).abs().max()) <= 1e-6, i
    ctx.close()


def test_server_admission_by_pool_memory(oracle):
    """A pool that holds one request's bricks at a time: requests are admitted
    one by one as bricks are released, and still render correctly."""
    import torch
    import livre_gb300 as lv
    vi = lv.VolumeInformation(128, 32, 1)
    ovol = oracle.volume(128, 32, 1)
    cams = [lv.orbit_camera(k, 4, vi.world_size, 48, 48, radius_scale=1.0) for k in range(4)]
    sizes = [len(oracle.select_visible(ovol, mv, pr, 48, 0.7)[0]) for mv, pr in cams]
    slot = vi.slot_bytes
    ctx = lv.Context(0, pool_bytes=max(sizes) * slot + slot)
    v = ctx.blob_volume(vi, 9, 4)
    tf = ctx.transfer_function(lv.linear_ramp_tf())
    reqs = [(v, tf, ctx.render_desc(mv, pr, 48, 48, sse=0.7)) for mv, pr in cams]
    srv = lv.Server(ctx, mode=0, max_batch=4)
    outs = [torch.zeros((48, 48, 4), dtype=torch.float32, device="cuda") for _ in reqs]
    tickets = [srv.submit(a, b, c, o) for (a, b, c), o in zip(reqs, outs)]
    res = [srv.wait(t) for t in tickets]
    assert all(r["status"] == 0 for r in res)
    srv.close()
    ref = alone(ctx, reqs)
    for a, b in zip(ref, outs):
        assert float((a - b).abs().max()) <= 1e-6
    ctx.close()


def test_server_concurrent_submitters():
    import torch
    import livre_gb300 as lv
    ctx = lv.Context(0, pool_bytes=512 << 20)
    vols, tfs, reqs = scene(ctx, lv, seed=3, n=24)
    srv = lv.Server(ctx, mode=0, max_batch=16)
    outs = [torch.zeros((d.height, d.width, 4), dtype=torch.float32, device="cuda")
            for _, _, d in reqs]
    tickets = [None] * len(reqs)

    def worker(lo, hi):
        for i in range(lo, hi):
            v, t, d = reqs[i]
            tickets[i] = srv.submit(v, t, d, outs[i])

    th = [threading.Thread(target=worker, args=(k * 6, k * 6 + 6)) for k in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    res = [srv.wait(t) for t in tickets]
    assert all(r["status"] == 0 for r in res)
    assert srv.counters()["completed"] == len(reqs)
    srv.close()
    ref = alone(ctx, reqs)
    for a, b in zip(ref, outs):
        assert float((a - b).abs().max()) <= 1e-6
    ctx.close()
