import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def native():
    """The built C-ABI library (loads without touching a GPU)."""
    import spinoza_gb300
    from spinoza_gb300 import _native

    spinoza_gb300.build()
    return _native.load()


@pytest.fixture(scope="session")
def gpu(native):
    """The library on a visible CUDA device; GPU tests fail loudly without one."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return native
