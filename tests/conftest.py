import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the library; on a GPU run a failure is an error."""
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    from mnpbem_gb300 import build, _lib
    build.build()
    return _lib.load()
