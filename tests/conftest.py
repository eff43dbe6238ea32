import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running parity case")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def nfx_lib():
    """The native library; building it needs nvcc, loading it needs no GPU."""
    from nofluidx3d_gb300 import _lib

    return _lib.load()
