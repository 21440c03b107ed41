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


# Routines beyond the solve path itself (refinement with error bounds,
# condition estimation, the expert driver, the inverse, Cholesky, complex LU) run after
# the solve-path tests, so that a run
# stopped at its first failure (-x) still reports the solve path in full.
_AFTER_SOLVE_PATH = {"test_gpu_refine.py": 1, "test_gpu_condest.py": 2, "test_gpu_svx.py": 3, "test_gpu_getri.py": 4,
                     "test_gpu_chol.py": 5, "test_gpu_zlu.py": 6}


# The allocation-free entry point's test file comes after everything else,
# so a run stopped at its failure has already run every other test.
_LAST = "test_zz_no_alloc.py"


def pytest_collection_modifyitems(session, config, items):
    items.sort(key=lambda it: (it.fspath.basename == _LAST, _AFTER_SOLVE_PATH.get(it.fspath.basename, 0)))
