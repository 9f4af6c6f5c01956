import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def capi():
    """The CUDA library (built if stale).  GPU tests only."""
    from lbmcl_gb300 import build, capi as _capi
    build.build_library()
    if not _have_gpu():
        pytest.fail("a GPU test ran without a visible CUDA device")
    return _capi


@pytest.fixture(scope="session")
def libonly():
    """The CUDA library loaded without touching the GPU (CPU tests)."""
    from lbmcl_gb300 import build, capi as _capi
    build.build_library()
    _capi.lib()
    return _capi
