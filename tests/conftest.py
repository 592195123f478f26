import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """Builds (if needed) and loads liblivre_gb300.so."""
    from livre_gb300 import build
    build.build()
    from livre_gb300 import _abi
    return _abi.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_ctx(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import livre_gb300 as lv
    ctx = lv.Context(0, pool_bytes=2 << 30)
    yield ctx
    ctx.close()


def compile_against_include(src, out, shared):
    """g++ of a C++ file written against include/ (the Livre-compatible
    headers), linked to liblivre_gb300."""
    from livre_gb300 import _abi
    libdir = os.path.dirname(_abi.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), src, "-o", out,
           "-L", libdir, "-llivre_gb300", "-Wl,-rpath," + libdir]
    if shared:
        cmd[1:1] = ["-fPIC", "-shared"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="session")
def checker_plugin(native, tmp_path_factory):
    """tests/plugins/checker_source.cpp built as libLivreCheckerSource.so and
    loaded into this process by lv.load_plugins (its static registerer adds
    the checker:// source). Returns (directory, loaded, loaded again)."""
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    import livre_gb300 as lv
    d = tmp_path_factory.mktemp("plugins")
    compile_against_include(os.path.join(ROOT, "tests", "plugins", "checker_source.cpp"),
                            str(d / "libLivreCheckerSource.so"), shared=True)
    # a library that the pattern does not match is left alone
    shutil.copy(d / "libLivreCheckerSource.so", d / "libUnrelated.so")
    first = lv.load_plugins(str(d))
    again = lv.load_plugins(str(d))
    return d, first, again
