"""ctypes loaders for the CPU oracle (oracle/liboracle.so) and, on the
development machine only, the reference built from source
(oracle/_ref/libpxref.so).  Test infrastructure: the GB300 package never
imports this module."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libpxref.so")

_oracle = None
_ref = None


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def oracle():
    global _oracle
    if _oracle is None:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        _oracle = ctypes.CDLL(ORACLE_SO)
        _oracle.orc_bp_create.restype = ctypes.c_void_p
        _oracle.orc_bp_release.argtypes = [ctypes.c_void_p]
    return _oracle


def reference():
    """The reference library, or None where it was not built (GPU machines)."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        _ref = ctypes.CDLL(REF_SO)
        _ref.pxref_bp_create.restype = ctypes.c_void_p
        _ref.pxref_bp_release.argtypes = [ctypes.c_void_p]
    return _ref


class CpuBroadPhase:
    """Same call pattern for the oracle ("orc") and the reference ("pxref")."""

    def __init__(self, which="orc", discard_sk=0, discard_kk=0):
        self.L = oracle() if which == "orc" else reference()
        self.pre = which
        self.h = ctypes.c_void_p(getattr(self.L, self.pre + "_bp_create")(discard_sk, discard_kk))

    def update(self, fr):
        cap = int(fr["capacity"])
        bounds = np.ascontiguousarray(fr["bounds"], np.float32)
        maxp = 1 << 20
        oc = np.zeros(2 * maxp, np.uint32)
        ol = np.zeros(2 * maxp, np.uint32)
        nc = np.zeros(1, np.uint32)
        nl = np.zeros(1, np.uint32)
        c = np.ascontiguousarray(fr["created"], np.uint32)
        u = np.ascontiguousarray(fr["updated"], np.uint32)
        r = np.ascontiguousarray(fr["removed"], np.uint32)
        g = np.ascontiguousarray(fr["groups"], np.uint32)
        d = np.ascontiguousarray(fr["distances"], np.float32)
        rc = getattr(self.L, self.pre + "_bp_update")(self.h, _p(c), len(c), _p(u), len(u), _p(r), len(r), _p(bounds), _p(g),
                                                      _p(d), cap, _p(oc), maxp, _p(nc), _p(ol), maxp, _p(nl))
        assert rc == 0, "pair buffer overflow"
        return oc[: 2 * nc[0]].reshape(-1, 2).copy(), ol[: 2 * nl[0]].reshape(-1, 2).copy()

    def release(self):
        if self.h:
            getattr(self.L, self.pre + "_bp_release")(self.h)
            self.h = None
