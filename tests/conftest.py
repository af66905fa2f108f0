"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and call the
CUDA path through the C ABI; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def rg():
    import raccoongpurender_gb300 as rg
    rg.load_library()
    return rg


@pytest.fixture(scope="session")
def po():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


def bits(a: np.ndarray) -> np.ndarray:
    """float32 array viewed as uint32, for bit-exact comparisons."""
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
