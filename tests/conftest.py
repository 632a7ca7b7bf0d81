import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs libqhg_gpu.so)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def has_cuda_device() -> bool:
    try:
        import ctypes
        lib = ctypes.CDLL("libcudart.so")
    except OSError:
        lib = None
    if lib is None:
        try:
            import torch
            return torch.cuda.is_available()
        except Exception:
            return False
    n = ctypes.c_int(0)
    return lib.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def gpu_lib():
    """libqhg_gpu.so, built if needed.  GPU tests fail (not skip) without it."""
    from qhg4_gb300.build import build
    from qhg4_gb300.gpu import load_library
    build()
    return load_library()
