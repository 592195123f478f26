"""A C++ host renders through the reference's downstream interface on the
GPU: livre::RenderPipeline::render with a livre::gb300::CudaRayCastRenderer
(tests/plugins/pipeline_check.cpp, compiled with -Werror against include/).
Its frame equals the oracle's within 1/255; the hooks run start, render,
end; the bricks it was handed are in the reference's distance order; the
availability, histogram and redraw filters report the frame; interacting
(idle false) renders the coarsest allowed level only."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def build(tmp_path):
    from livre_gb300 import _abi
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(_abi.LIB_PATH)
    exe = str(tmp_path / "pipeline_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(os.path.dirname(HERE), "include"),
                        "-I", os.path.join(cuda, "include"),
                        os.path.join(HERE, "plugins", "pipeline_check.cpp"), "-o", exe,
                        "-L", libdir, "-llivre_gb300", "-Wl,-rpath," + libdir,
                        "-L", os.path.join(cuda, "lib64"), "-lcudart",
                        "-Wl,-rpath," + os.path.join(cuda, "lib64")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_render_pipeline_with_cuda_renderer(native, oracle, tmp_path):
    import torch
    if not torch.cuda.is_available() or shutil.which("g++") is None:
        pytest.skip("needs a CUDA device and g++")
    import livre_gb300 as lv
    exe = build(tmp_path)
    W, H = 96, 80
    ovol = oracle.volume(128, 32, 1)
    mv, proj = lv.orbit_camera(3, 8, tuple(ovol.world_size), W, H, radius_scale=1.2)
    tf = lv.gaussian_peaks_tf(256, seed=5)
    view = tmp_path / "view.bin"
    np.concatenate([np.asarray(mv, np.float32).reshape(16), np.asarray(proj, np.float32).reshape(16),
                    tf.ravel()]).astype(np.float32).tofile(view)
    out = tmp_path / "frame.raw"
    r = subprocess.run([exe, str(view), str(W), str(H), str(out)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert lines["hooks"] == "start render end"
    f = lines["visible"].split()
    visible, available, not_available = int(f[0]), int(f[2]), int(f[4])
    rendered, samples, spr = int(f[6]), int(f[8]), int(f[10])
    assert spr == 256
    ids, _ = oracle.select_visible(ovol, mv, proj, H, 1.0)
    assert visible == len(ids) and available == len(ids) and not_available == 0
    assert rendered == len(ids)
    ordered = [int(x) for x in lines["order"].split()]
    assert sorted(ordered) == sorted(int(i) for i in ids)
    # the reference's order: ascending eye-space distance of the brick centres
    m = np.asarray(mv, np.float64).reshape(4, 4).T
    def dist(i):
        b = oracle.world_box(ovol, i).astype(np.float64)
        c = np.append((b[:3] + b[3:]) / 2, 1.0)
        return float(np.linalg.norm((m @ c)[:3]))
    d = [dist(i) for i in ordered]
    assert all(d[k] <= d[k + 1] + 1e-6 for k in range(len(d) - 1))
    filt = lines["filters"].split()
    assert filt[1] == "0" and filt[3] == "1" and filt[5] == "42" and int(filt[7]) > 0
    # the frame against the oracle
    img = np.fromfile(out, np.float32).reshape(H, W, 4)
    bp = oracle.blob_params(8, 1, 0, 1)
    bricks = np.stack([oracle.blob_brick(ovol, bp, int(i)) for i in ids])
    ref, ns = oracle.raycast(ovol, 1, ids, bricks, tf,
                             oracle.make_view(mv, proj, W, H, 256, early_exit=0.999))
    assert np.abs(img - ref).max() <= 1.0 / 255.0
    assert abs(samples - ns) <= max(8, ns // 2000)
    # interaction renders the minimum LOD only
    inter = lines["interacting"].split()  # visible N max_level L
    assert int(inter[1]) >= 1 and inter[3] == "0"
