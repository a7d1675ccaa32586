import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def lib():
    from muontomography_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def gpu(lib):
    import ctypes

    cudart = None
    n = ctypes.c_int(0)
    try:
        import torch  # device presence only; the kernels are ours

        if not torch.cuda.is_available():
            pytest.fail("GPU test run without a visible CUDA device")
    except ImportError:
        pass
    return True
