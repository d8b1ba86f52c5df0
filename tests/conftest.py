import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "geophyinv.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine")
    config.addinivalue_line("markers", "slow: long CPU oracle runs")


@pytest.fixture(scope="session")
def engine():
    """The CUDA engine; GPU tests fail (not skip) when it is missing."""
    import torch

    assert torch.cuda.is_available(), "GPU test needs CUDA"
    from geophyinv_gb300 import _lib

    return _lib.load()
