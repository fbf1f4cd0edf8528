import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if stale) and returns the path of the in-tree CUDA library."""
    from cusat_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cusat_gb300 import build
    build.build()
    torch.cuda.init()
    return torch
