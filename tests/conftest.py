import os
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
