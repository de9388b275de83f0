import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    """The built CUDA library (built in-tree on first use)."""
    from zquatev_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(lib):
    if not _cuda_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return lib
