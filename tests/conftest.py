import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-sfft_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgsfft.so")


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (built on first use)."""
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def G():
    """The GPU engine binding; builds libgsfft.so if needed."""
    import gsfft
    if not os.path.exists(gsfft.LIB_PATH):
        gsfft.build()
    gsfft.lib()
    return gsfft


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
