"""Data-source plugins written the reference's way.

tests/plugins/checker_source.cpp is a livre::DataSourcePlugin registered with
lunchbox::PluginRegisterer, compiled here against include/ (the
source-compatible headers) into libLivreCheckerSource.so and loaded the way
DataSource::loadPlugins does (livre/data/DataSource.cpp:58-62).
tests/plugins/datasource_check.cpp restates the reference's data-source test
(tests/data/dataSource.cpp:31-64) against the same headers.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CHECKER = "checker://#128,96,64,32"

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


@pytest.fixture(scope="module")
def plugin_dir(checker_plugin):
    return checker_plugin


def checker_brick(info, node_id):
    """The checker plugin's brick of node_id, restated in numpy."""
    import livre_gb300 as lv
    nid = lv.NodeId(int(node_id))
    s = 1 << (info.depth - 1 - nid.level)
    block = info.block_size
    axes = []
    for a in range(3):
        lo = nid.position[a] * block[a]
        last = (info.voxels[a] + s - 1) // s - 1
        g = np.clip(lo + np.arange(info.max_block[a]) - 1, 0, last)
        axes.append((g * s + s // 2) // 16)
    fz, fy, fx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    v = 40 + 170 * ((fx + fy + fz) & 1)
    if info.dtype == lv.DT_UINT16:
        return (v * 257).astype(np.uint16).view(np.uint8).reshape(-1)
    return v.astype(np.uint8).reshape(-1)


def test_plugins_load_once_by_pattern(plugin_dir):
    _, first, again = plugin_dir
    assert first == 1  # libUnrelated.so does not match Livre.*Source
    assert again == 0


def test_plugin_handles_and_describes(plugin_dir):
    import livre_gb300 as lv
    assert lv.source_handles(CHECKER)
    assert lv.source_handles("mem://")
    assert lv.source_handles("volume.nrrd")  # no scheme: RawDataSource by extension
    assert not lv.source_handles("nosuchscheme://volume")
    text = lv.source_descriptions()
    assert text.startswith("checkerboard test volume")
    assert "mem://" in text


def test_plugin_volume_information(plugin_dir):
    import livre_gb300 as lv
    vi = lv.probe_source(CHECKER)
    ref = lv.VolumeInformation((128, 96, 64), 32, overlap=1, dtype=lv.DT_UINT8)
    assert vi.voxels == (128, 96, 64)
    assert vi.max_block == (34, 34, 34)
    assert vi.overlap == (1, 1, 1)
    assert vi.dtype == lv.DT_UINT8
    assert (vi.depth, vi.root_blocks) == (ref.depth, ref.root_blocks)
    assert vi.world_size == ref.world_size
    assert lv.probe_source(CHECKER + ",16").dtype == lv.DT_UINT16


@pytest.mark.parametrize("bits", [8, 16])
def test_plugin_bricks_through_the_host_source(plugin_dir, bits):
    import livre_gb300 as lv
    uri = CHECKER + (",16" if bits == 16 else "")
    with lv.DataSource(uri) as src:
        info = src.info
        for nid in info.all_nodes():
            got = src.get_data(nid)
            assert got is not None and got.size == info.brick_bytes
            np.testing.assert_array_equal(got, checker_brick(info, nid))
        assert src.get_data(lv.NodeId()) is None
        assert src.get_data(lv.NodeId(0, (9, 0, 0))) is None


def test_reference_datasource_checks_compile_and_pass(plugin_dir, tmp_path):
    d, _, _ = plugin_dir
    from conftest import compile_against_include
    exe = str(tmp_path / "datasource_check")
    compile_against_include(os.path.join(HERE, "plugins", "datasource_check.cpp"), exe, shared=False)
    env = dict(os.environ, LD_LIBRARY_PATH=str(d))
    r = subprocess.run([exe, "mem://#1024,1024,512,32", "checker://#1024,1024,512,32"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failure(s)" in r.stdout


def test_unregistered_source_is_not_found(native):
    import ctypes as C
    from livre_gb300 import _abi
    L = _abi.lib()
    handles = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p)(lambda u, uri: 0)
    opener = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p)(lambda *a: 0)
    hp = C.cast(handles, C.c_void_p)
    op = C.cast(opener, C.c_void_p)
    assert L.lv_register_source(hp, op, None, b"never handles") == _abi.LV_OK
    assert L.lv_unregister_source(hp, op) == _abi.LV_OK
    assert L.lv_unregister_source(hp, op) == _abi.LV_ENOTFOUND
    assert L.lv_register_source(None, op, None, None) == _abi.LV_EINVAL


def test_host_datasource_built_in_sources(native, tmp_path):
    """lv_source_open without a device: mem:// bricks (the known answer of
    MemoryDataSource::computeData) and a raw:// file read back as written."""
    import math
    import livre_gb300 as lv
    with lv.DataSource("mem://?datatype=uint16#256,256,256,32") as src:
        assert src.info.depth == 4 and src.info.max_block == (40, 40, 40)
        n = lv.NodeId(2, (1, 2, 3), 9)
        b = n.id.to_bytes(8, "little")
        want = int(float((b[0] ^ b[1] ^ b[2] ^ b[3]) + 16) + 127.0 * math.sin((9 + 1) / 200.0))
        assert (src.get_data(n).view(np.uint16) == want).all()
    data = (np.arange(12 * 10 * 8, dtype=np.uint32) * 7919 % 65536).astype(np.uint16)
    path = tmp_path / "ramp.raw"
    data.tofile(path)
    with lv.DataSource("raw://%s#12,10,8,uint16" % path) as src:
        assert src.info.voxels == (12, 10, 8) and src.info.depth == 1
        assert (src.get_data(lv.NodeId(0, (0, 0, 0))).view(np.uint16) == data).all()
    with lv.DataSource(str(tmp_path / "ramp.raw") + "#12,10,8,uint16") as src:
        assert src.info.voxels == (12, 10, 8)  # no scheme: a .raw path


def test_source_errors(native, tmp_path):
    import livre_gb300 as lv
    with pytest.raises(lv.LivreError):
        lv.DataSource("nosuchscheme://volume")
    with pytest.raises(lv.LivreError):
        lv.DataSource("raw://%s#4,4,4" % (tmp_path / "missing.raw"))
    with pytest.raises(lv.LivreError):
        lv.DataSource("mem://?datatype=complex64")
    with pytest.raises(lv.LivreError):
        lv.load_plugins(str(tmp_path), pattern="(unbalanced")
    assert lv.load_plugins(str(tmp_path / "does-not-exist")) == 0
