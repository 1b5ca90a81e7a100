import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def built_lib():
    """Build libppf_gb300.so (nvcc) once per session; returns its path."""
    from pyphasefield_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyphasefield_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)
