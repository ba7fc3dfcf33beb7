import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import ctypes
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        else:
            return False
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libocpx_gb300.so; GPU tests fail loudly
    when no device is present instead of falling back to anything."""
    from opencaeporox_gb300 import build
    build.build()
    from opencaeporox_gb300 import fim
    if not _cuda_available():
        pytest.fail("no CUDA device visible to a GPU-marked test")
    return fim.load_library()
