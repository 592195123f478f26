"""The downstream interface headers (livre::Renderer, Frustum, RenderParams,
RenderPipeline, gb300::CudaRayCastRenderer) compile with -Werror against
include/ alone, and their host-side logic holds (CPU only): the stage hooks
of Renderer::render (livre/core/render/Renderer.cpp:33-47), frustum limits,
the matrix inverse, the brick distance order (RayCastRenderer.cpp:57-81)
and the render description with the interaction clamp
(RenderPipeline.cpp:71-74)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT, compile_against_include


def test_renderer_interface_host_logic(native, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    exe = str(tmp_path / "renderer_stages")
    compile_against_include(os.path.join(ROOT, "tests", "plugins", "renderer_stages.cpp"), exe,
                            shared=False)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
