import ctypes
import ctypes.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def _device_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0:
            return n.value
        return 0
    return 0


@pytest.fixture(scope="session")
def gpu():
    """The product library on a machine with a GPU.  Missing library on a GPU machine fails."""
    if _device_count() == 0:
        pytest.skip("no CUDA device on this machine")
    from wumingpic2d_gb300 import _native

    return _native.lib()
