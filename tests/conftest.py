import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, loaded; fails (not skips) when it cannot load on a GPU machine."""
    import torch
    import lapack_gb300 as g
    assert torch.cuda.is_available(), "GPU test run without a GPU"
    g.lib()
    return g


@pytest.fixture()
def exact_mode(gpu):
    old = gpu.set_option("exact", 1)
    yield
    gpu.set_option("exact", old)
