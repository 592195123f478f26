"""URI data sources (mem://, raw://) and brick histograms against the
reference's known answers:
  tests/data/dataSource.cpp:39-64    mem://#1024,1024,512,32 has depth 5
  tests/lib/cache.cpp:40-135         getData bytes of the first child of the
                                     root; its histogram has max bin 17 with
                                     2^24 counts, and summing it twice gives 2^25
  tests/data/rawDatasource.cpp:40-83 the 41^3 nucleon volume is one brick
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NUCLEON = os.path.join(GOLDEN, "nucleon.raw")


@pytest.fixture
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    c = lv.Context(0, pool_bytes=256 << 20)
    yield c
    c.close()


def test_memory_source_and_histogram_known_answer(ctx):
    import livre_gb300 as lv
    v = ctx.open_volume("mem://#1024,1024,512,32")
    assert v.info.depth == 5 and v.info.comp_count == 1
    assert v.info.max_block == (40, 40, 40) and v.info.overlap == (4, 4, 4)
    child = lv.NodeId(0, (0, 0, 0)).get_children()[0]
    data = v.get_data(child.id)
    assert data.size == 40 ** 3 and (data == 17).all()
    hist = v.histogram([child.id], 256, (0.0, 255.0))
    assert hist[17] == 1 << 24 and int(hist.sum()) == 1 << 24
    assert int(np.argmin(hist)) == 0 and int(np.argmax(hist)) == 17
    twice = v.histogram([child.id, child.id], 256, (0.0, 255.0))
    assert twice[17] == 1 << 25 and int(twice.sum()) == 1 << 25
    assert v.get_data(lv.NodeId().id) is None  # invalid id: no data
    v.close()


def test_memory_source_types_and_time_steps(ctx):
    import math
    import livre_gb300 as lv
    v = ctx.open_volume("mem://?datatype=uint16#256,256,256,32")
    n = lv.NodeId(2, (1, 2, 3), 9)
    b = n.id.to_bytes(8, "little")
    want = int(float((b[0] ^ b[1] ^ b[2] ^ b[3]) + 16) + 127.0 * math.sin((9 + 1) / 200.0))
    data = v.get_data(n.id).view(np.uint16)
    assert (data == want).all()
    v.close()


def test_unknown_scheme_rejected(ctx):
    import livre_gb300 as lv
    with pytest.raises(lv.LivreError):
        ctx.open_volume("uvf://nowhere.uvf")


def test_raw_and_nrrd_sources(ctx, tmp_path):
    import livre_gb300 as lv
    raw = np.fromfile(NUCLEON, np.uint8)
    for uri in ("raw://%s#41,41,41,uint8" % NUCLEON, None):
        if uri is None:
            hdr = tmp_path / "nucleon.nrrd"
            hdr.write_text("NRRD0001\ncontent: nucleon\ndimension: 3\ntype: uchar\n"
                           "sizes: 41 41 41\nspacings: 1 1 1\ndatafile: %s\nencoding: raw\n"
                           % NUCLEON)
            uri = "raw://%s" % hdr
        v = ctx.open_volume(uri)
        assert v.info.depth == 1 and v.info.voxels == (41, 41, 41)
        assert v.info.max_block == (41, 41, 41) and v.info.overlap == (0, 0, 0)
        assert (v.get_data(lv.NodeId(0, (0, 0, 0)).id) == raw).all()
        v.close()


def test_raw_output_conversion(ctx, tmp_path):
    data = (np.arange(8 * 8 * 8, dtype=np.uint32) * 7919).astype(np.uint16)
    p = tmp_path / "ramp.raw"
    data.tofile(p)
    v = ctx.open_volume("raw://%s?output=uint8#8,8,8,uint16" % p)
    got = v.get_data(0)
    assert (got == (data >> 8).astype(np.uint8)).all()
    v.close()


@pytest.mark.parametrize("filt", [0, 1])
def test_nucleon_render_matches_oracle(ctx, oracle, filt):
    """One brick without overlap: the clamp-to-edge sampling path."""
    import livre_gb300 as lv
    v = ctx.open_volume("raw://%s#41,41,41,uint8" % NUCLEON)
    ovol = oracle.volume(41, 41, 0)
    tf_rgba = lv.default_transfer_function()
    tf = ctx.transfer_function(tf_rgba)
    mv, proj = lv.orbit_camera(3, 8, v.info.world_size, 80, 64, radius_scale=1.0)
    img = ctx.render(v, tf, ctx.render_desc(mv, proj, 80, 64, sse=1.0, filt=filt,
                                            step_policy=lv.STEP_REFERENCE)).cpu().numpy()
    st = ctx.last_stats()
    assert st["n_rendered"] == 1 and st["samples_per_ray"] == 512
    raw = np.fromfile(NUCLEON, np.uint8)
    view = oracle.make_view(mv, proj, 80, 64, 512, filt=filt)
    ref, ns = oracle.raycast(ovol, 1, [0], raw[None, :], tf_rgba, view)
    assert ns > 0
    assert np.abs(img - ref).max() <= 1.0 / 255.0
    # one brick: the per-brick shader transcription (FP64, its own ray
    # geometry) agrees too, sample counts within a face sample or two
    shader, ns_shader = oracle.raycast(ovol, 1, [0], raw[None, :], tf_rgba, view, mode=1)
    assert np.abs(img - shader).max() <= 1.0 / 255.0
    assert abs(int(st["n_samples"]) - ns_shader) <= max(8, ns_shader // 20000)
    tf.close()
    v.close()


def test_blob_histogram_matches_numpy(ctx, oracle):
    import livre_gb300 as lv
    vi = lv.VolumeInformation(96, 32, 1, dtype=lv.DT_UINT16)
    ovol = oracle.volume(96, 32, 1)
    v = ctx.blob_volume(vi, 6, 3, noise=2)
    ids = [lv.NodeId(1, (1, 0, 1)).id, lv.NodeId(0, (0, 0, 0)).id]
    acc, per = v.histogram(ids, 1024, (0.0, 65535.0), per_brick=True)
    bp = oracle.blob_params(6, 3, 2, 2)
    want_acc = np.zeros(1024, np.uint64)
    for k, i in enumerate(ids):
        b = oracle.blob_brick(ovol, bp, i).reshape(34, 34, 34)[1:33, 1:33, 1:33]
        level = i & 0xF
        scale = (2 ** (vi.depth - 1 - level)) ** 3
        bins = np.clip(np.floor((b.astype(np.float32) - np.float32(0.0)) *
                                np.float32(1023.0 / 65535.0)), 0, 1023).astype(np.int64)
        h = np.bincount(bins.ravel(), minlength=1024).astype(np.uint64) * np.uint64(scale)
        assert (per[k] == h).all()
        want_acc += h
    assert (acc == want_acc).all()
    v.close()
