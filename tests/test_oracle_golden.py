"""The CPU oracle and the host-side product logic against the reference's own
golden vectors and known-answer tests (no GPU needed).

Sources (BlueBrain/Livre):
  tests/data/lodSelection.cpp:70-207      golden visible NodeId sets
  tests/data/volumeInformation.cpp:57-106 fillRegularVolumeInfo cases
  tests/data/dataSource.cpp:39-64         depth of mem://#1024,1024,512,32
  tests/data/rawDatasource.cpp:40-83      depth of the 41^3 nucleon volume
  tests/core/transferFunction.cpp:53-72   LUT of tf_f.1dt, default TF fallback
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def lod_golden():
    return json.load(open(os.path.join(GOLDEN, "lod_selection.json")))


def golden_volume(oracle):
    # mem://#4096,4096,4096,256: MemoryDataSource adds overlap 4
    # (livre/data/MemoryDataSource.cpp:66,103-105)
    return oracle.volume(4096, 256, 4)


@pytest.mark.parametrize("case", range(8))
def test_lod_selection_golden(oracle, case):
    g = lod_golden()
    c = g["cases"][case]
    vol = golden_volume(oracle)
    ids, _ = oracle.select_visible(vol, g["mv"], g["proj"], c["window_height"], c["sse"],
                                   c["min_lod"], c["max_lod"])
    assert sorted(int(i) for i in ids) == c["expected"]


def test_lod_selection_levels_pinned(oracle):
    """maxLOD == minLOD cases keep every id at that level (lodSelection.cpp:177-207)."""
    g = lod_golden()
    vol = golden_volume(oracle)
    for lvl in (0, 1):
        ids, _ = oracle.select_visible(vol, g["mv"], g["proj"], 512, 1.0, lvl, lvl)
        assert all(int(i) & 0xF == lvl for i in ids)


VOLINFO_CASES = [
    # voxels, block, overlap -> depth, root blocks, wspv, world size
    ((2048, 2048, 2048), 64, 0, 6, (1, 1, 1), 1 / 2048, (1.0, 1.0, 1.0)),
    ((2048, 2099, 2048), 64, 0, 6, (1, 2, 1), 1 / 2099, (2048 / 2099, 1.0, 2048 / 2099)),
    ((2048, 2037, 2048), 64, 0, 6, (1, 1, 1), 1 / 2048, (1.0, 2037 / 2048, 1.0)),
    ((2048, 2049, 2048), 64, 0, 6, (1, 1, 1), 1 / 2049, (2048 / 2049, 1.0, 2048 / 2049)),
    ((1024, 1024, 512), 32, 4, 5, None, None, None),
    ((41, 41, 41), 41, 0, 1, (1, 1, 1), None, None),
    ((4096, 4096, 4096), 256, 4, 5, (1, 1, 1), None, None),
]


@pytest.mark.parametrize("case", VOLINFO_CASES)
def test_volume_information_oracle(oracle, case):
    voxels, block, overlap, depth, roots, wspv, ws = case
    v = oracle.volume(voxels, block, overlap)
    assert v.depth == depth
    if roots:
        assert tuple(v.root_blocks) == roots
    if wspv:
        assert v.wspv == np.float32(1.0) / np.float32(max(voxels))
        assert tuple(np.float32(x) for x in v.world_size) == tuple(np.float32(x) for x in ws)


@pytest.mark.parametrize("case", VOLINFO_CASES)
def test_volume_information_product(native, oracle, case):
    """lv_fill_regular_volume_info (host code of the library) equals the oracle."""
    import livre_gb300 as lv
    voxels, block, overlap = case[:3]
    p = lv.VolumeInformation(voxels, block, overlap)
    o = oracle.volume(voxels, block, overlap)
    assert p.depth == o.depth
    assert p.root_blocks == tuple(o.root_blocks)
    assert np.float32(p.world_space_per_voxel) == np.float32(o.wspv)
    assert p.world_size == tuple(o.world_size)


def test_default_volume_information():
    """VolumeInformation defaults (tests/data/volumeInformation.cpp:40-55)."""
    import livre_gb300 as lv
    p = lv.VolumeRendererParameters()
    assert (p.max_lod, p.min_lod, p.screen_space_error, p.samples_per_ray,
            p.max_gpu_cache_memory) == (9, 0, 4.0, 0, 3072)


def test_tf_lut_golden(oracle):
    d = json.load(open(os.path.join(GOLDEN, "tf_f.json")))
    vals = np.array(d["rgba"], np.float32).reshape(d["n"], 4)
    expected = (vals * np.float32(255.0)).astype(np.uint8)
    assert (oracle.tf_lut(vals) == expected).all()
    import livre_gb300 as lv
    assert (lv.TransferFunction1D(vals).get_lut() == expected).all()


def test_tf_file_loader(tmp_path):
    import livre_gb300 as lv
    d = json.load(open(os.path.join(GOLDEN, "tf_f.json")))
    p = tmp_path / "tf_f.1dt"
    rows = np.array(d["rgba"], np.float32).reshape(-1, 4)
    p.write_text("%d\n" % len(rows) + "\n".join(" ".join(repr(float(x)) for x in r) for r in rows))
    tf = lv.TransferFunction1D.from_file(str(p))
    assert (tf.rgba == rows).all()
    # inexistent file / wrong extension -> default TF (transferFunction.cpp:64-72)
    assert (lv.TransferFunction1D.from_file(str(tmp_path / "none.1dt")).get_lut()
            == lv.TransferFunction1D().get_lut()).all()


def test_default_tf_product_matches_oracle(oracle):
    import livre_gb300 as lv
    assert (lv.default_transfer_function() == oracle.default_tf()).all()


def test_nodeid_layout_and_children(oracle):
    import livre_gb300 as lv
    n = lv.NodeId(2, (1, 2, 3), 5)
    assert n.level == 2 and n.position == (1, 2, 3) and n.time_step == 5
    assert n.id == 2 | (1 << 4) | (2 << 18) | (3 << 32) | (5 << 46)
    ch = n.get_children()
    assert [c.id for c in ch] == oracle.children(n.id)
    assert ch[0].position == (2, 4, 6) and ch[1].position == (2, 4, 7)
    assert ch[4].position == (3, 4, 6)
    assert all(c.get_parent() == n for c in ch)
    assert not lv.NodeId().is_valid()
    assert lv.NodeId(0, (0, 0, 0)).get_parent() == lv.NodeId()
    assert [p.level for p in ch[7].get_parents()] == [2, 1, 0]


def test_exp_polynomial_accuracy(oracle):
    xs = np.linspace(-18.0, 0.0, 2001)
    got = np.array([oracle.exp_neg(x) for x in xs])
    ref = np.exp(xs.astype(np.float32).astype(np.float64))
    assert np.max(np.abs(got - ref) / ref) < 3e-6


def test_blob_point_sampling(oracle):
    """A level-L voxel is the blob function at its centre, in finest voxels."""
    vol = oracle.volume(64, 16, 1)
    bp = oracle.blob_params(8, seed=7)
    brick = oracle.blob_brick(vol, bp, 1 | (1 << 4))  # level 1, x = 1
    N = vol.max_block[0]
    b = brick.reshape(N, N, N)  # z, y, x
    # local voxel (i, j, k) = level-1 coord (16 - 1 + i, -1 + j, -1 + k) clamped
    i, j, k = 5, 6, 7
    g = (16 + i - 1, j - 1, k - 1)
    s = 2.0 ** (vol.depth - 1 - 1)
    v = oracle.lib().or_blob_value(vol, bp, (g[0] + 0.5) * s, (g[1] + 0.5) * s, (g[2] + 0.5) * s)
    q = int(np.floor(np.float32(min(max(v, 0.0), 1.0)) * np.float32(255.0) + np.float32(0.5)))
    assert b[k, j, i] == q
