import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and libpdfs in-tree once per session."""
    from oracle import oracle as O
    from pdfs_gb300 import build as B
    O.build(ref=False)
    B.build()
    yield


def have_gpu() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so.13")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False
