import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the tahoe_gb300 kernels)")


def cuda_available():
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        if hasattr(rt, "cudaGetDeviceCount"):
            n = ctypes.c_int(0)
            return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
        n = ctypes.c_int(0)
        return rt.cuInit(0) == 0 and rt.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
