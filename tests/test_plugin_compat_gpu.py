"""A volume served by a data-source plugin (tests/plugins/checker_source.cpp,
registered through lunchbox::PluginRegisterer) rendered on the device and
checked against the oracle ray cast of the same bricks.

Tolerance: max per-channel |GPU - oracle| <= 1/255 (FP32 kernel, FP64 oracle).
"""
import numpy as np
import pytest

from test_plugin_compat import CHECKER, checker_brick

pytestmark = pytest.mark.gpu
TOL = 1.0 / 255.0


@pytest.mark.parametrize("bits", [8, 16])
def test_plugin_volume_renders_like_the_oracle(gpu_ctx, oracle, checker_plugin, bits):
    import livre_gb300 as lv
    uri = CHECKER + (",16" if bits == 16 else "")
    v = gpu_ctx.open_volume(uri)
    info = v.info
    dtype = 2 if bits == 16 else 1
    assert info.dtype == dtype and info.max_block == (34, 34, 34)
    # the pool is fed the plugin's bytes
    for nid in list(info.all_nodes())[:3]:
        np.testing.assert_array_equal(v.get_data(nid.id), checker_brick(info, nid))
    ovol = oracle.volume(info.voxels, 32, 1)
    tf_rgba = lv.linear_ramp_tf(256)
    tf = gpu_ctx.transfer_function(tf_rgba)
    W, H = 96, 80
    with lv.DataSource(uri) as src:
        for k in range(3):
            mv, proj = lv.orbit_camera(k, 8, info.world_size, W, H, radius_scale=1.2)
            img = gpu_ctx.render(v, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0,
                                                            step_policy=1)).cpu().numpy()
            st = gpu_ctx.last_stats()
            ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
            assert st["n_rendered"] == len(ids) > 0
            bricks = np.stack([src.get_data(int(i)) for i in ids])
            view = oracle.make_view(mv, proj, W, H, st["samples_per_ray"],
                                    range_hi=65535.0 if bits == 16 else 255.0)
            ref, ns = oracle.raycast(ovol, dtype, ids, bricks, tf_rgba, view)
            assert ns > 1000
            err = np.abs(img - ref).max()
            assert err <= TOL, (k, err)
    tf.close()
    v.close()


def test_cpp_host_renders_a_plugin_volume(gpu_ctx, checker_plugin, tmp_path):
    """A C++ program drives the C ABI alone (plugins, URI, lv_render, PNG), in
    its own process; its frame equals the frame rendered here, byte for byte."""
    import os
    import shutil
    import subprocess
    import livre_gb300 as lv
    from livre_gb300 import _abi
    from test_png import read_png
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if shutil.which("g++") is None or not os.path.isdir(os.path.join(cuda, "include")):
        pytest.skip("needs g++ and the CUDA headers")
    libdir = os.path.dirname(_abi.LIB_PATH)
    here = os.path.dirname(os.path.abspath(__file__))
    exe = str(tmp_path / "render_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(os.path.dirname(here), "include"),
                        "-I", os.path.join(cuda, "include"),
                        os.path.join(here, "plugins", "render_check.cpp"), "-o", exe,
                        "-L", libdir, "-llivre_gb300", "-Wl,-rpath," + libdir,
                        "-L", os.path.join(cuda, "lib64"), "-lcudart",
                        "-Wl,-rpath," + os.path.join(cuda, "lib64")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    W, H = 96, 72
    v = gpu_ctx.open_volume(CHECKER)
    mv, proj = lv.orbit_camera(2, 8, v.info.world_size, W, H, radius_scale=1.3)
    tf_rgba = lv.gaussian_peaks_tf(256, seed=5)
    view = tmp_path / "view.bin"
    # the camera as lv_render_desc holds it (lv.make_camera's layout)
    np.concatenate([np.asarray(mv, np.float32).reshape(16),
                    np.asarray(proj, np.float32).reshape(16),
                    tf_rgba.ravel()]).astype(np.float32).tofile(view)
    png = tmp_path / "frame.png"
    plugins_dir = str(checker_plugin[0])
    r = subprocess.run([exe, plugins_dir, CHECKER, str(view), str(W), str(H), str(png)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("visible ")
    tf = gpu_ctx.transfer_function(tf_rgba)
    img = gpu_ctx.render(v, tf, gpu_ctx.render_desc(mv, proj, W, H, sse=1.0,
                                                    early_exit=0.999))
    mine = gpu_ctx.to_rgba8(img).cpu().numpy()
    theirs = read_png(png.read_bytes())[::-1]  # the file is top row first
    assert theirs.shape == (H, W, 4)
    assert (theirs[..., 3] > 0).any()
    np.testing.assert_array_equal(theirs, mine)
    tf.close()
    v.close()
