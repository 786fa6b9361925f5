"""GB300-native rigid-body immediate-mode step (PhysX-compatible).

The compute path is ``libgbpx.so``: hand-written sm_103a CUDA kernels behind a
C ABI (``include/gbpx.h``).  This package is a thin ctypes mirror of the
reference's immediate-mode and PxBroadPhase interfaces.  There is no CPU
fallback: if the library is missing, importing the bindings raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbpx.so")
_lib = None

# Status codes (include/gbpx.h).
GBPX_OK = 0
_STATUS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "device buffer capacity exceeded",
    -4: "out of device memory",
    -5: "invalid call sequence",
    -6: "memory budget exceeded",
    -7: "bounded device wait timed out",
}


class GbpxError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__("%s failed: %s (%d)" % (what or "gbpx call", _STATUS.get(code, "unknown"), code))
        self.code = code


def lib():
    """Returns the loaded libgbpx.so; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbpx.so is not built (run physx_gb300.build.build()); "
                              "the GB300 path has no CPU fallback")
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def check(rc, what=""):
    if rc != GBPX_OK:
        raise GbpxError(rc, what)
    return rc


def set_device(device):
    """Selects the CUDA device used by subsequently created objects (one process per GPU)."""
    L = lib()
    L.gbpx_set_device.argtypes = [ctypes.c_int]
    check(L.gbpx_set_device(int(device)), "gbpx_set_device")
