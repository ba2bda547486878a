import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def mps():
    """The product library, built in-tree for sm_103a."""
    from mps_cuda_gb300 import build
    build.build()
    import mps_cuda_gb300
    mps_cuda_gb300._lib.load()
    return mps_cuda_gb300


@pytest.fixture(scope="session")
def orc():
    """The FP64 CPU oracle (checker only)."""
    from oracle import oracle
    oracle.build()
    oracle.load()
    return oracle


def has_gpu() -> bool:
    try:
        import ctypes
        cudart = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False
