import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C-ABI")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def gpu_lib():
    """The built libmisfit_gb (built on first use).  GPU tests fail loudly when
    it cannot be built or loaded."""
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    from misfit_gb300 import build, native
    build.build()
    return native.load_library()
