import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def gbpx_built():
    """Builds libgbpx.so in-tree (nvcc cross-compiles without a GPU)."""
    from physx_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda_device(gbpx_built):
    import ctypes
    import physx_gb300
    L = physx_gb300.lib()
    n = ctypes.c_int(0)
    L.gbpx_device_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    rc = L.gbpx_device_count(ctypes.byref(n))
    if rc != 0 or n.value < 1:
        pytest.fail("a GB300 GPU is required for -m gpu tests (no CUDA device visible)")
    return 0
