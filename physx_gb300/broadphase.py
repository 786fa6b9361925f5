"""PxBroadPhase (eABP) mirror over the GB300 broadphase.

Mirrors physx/include/PxBroadPhase.h: ``PxCreateBroadPhase`` (:629),
``PxBroadPhase::update`` / ``fetchResults`` (:576-602), the filter-group
helpers (:264-291), and ``PxBroadPhaseUpdateData`` (:312) argument meaning:
created/updated/removed handle lists, persistent user-owned bounds (6 floats
per handle: min xyz, max xyz), groups and distances indexed by handle.
"""
import ctypes

import numpy as np

from . import check, lib

_u32p = ctypes.POINTER(ctypes.c_uint32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _setup():
    L = lib()
    if getattr(L, "_bp_ready", False):
        return L
    L.gbpx_bp_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.gbpx_bp_release.argtypes = [ctypes.c_void_p]
    L.gbpx_bp_update.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                 ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_uint32]
    L.gbpx_bp_fetch_results.argtypes = [ctypes.c_void_p, ctypes.POINTER(_u32p), ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(_u32p), ctypes.POINTER(ctypes.c_uint32)]
    L.gbpx_bp_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    for f in ("gbpx_bp_dynamic_filter_group", "gbpx_bp_kinematic_filter_group"):
        getattr(L, f).argtypes = [ctypes.c_uint32]
        getattr(L, f).restype = ctypes.c_uint32
    L.gbpx_bp_static_filter_group.restype = ctypes.c_uint32
    L._bp_ready = True
    return L


def static_filter_group():
    return int(_setup().gbpx_bp_static_filter_group())


def dynamic_filter_group(i):
    return int(_setup().gbpx_bp_dynamic_filter_group(i))


def kinematic_filter_group(i):
    return int(_setup().gbpx_bp_kinematic_filter_group(i))


class BroadPhase:
    """GB300 ABP-compatible broadphase (``PxCreateBroadPhase(PxBroadPhaseDesc(eABP))``)."""

    def __init__(self, discard_static_vs_kinematic=False, discard_kinematic_vs_kinematic=False):
        L = _setup()
        h = ctypes.c_void_p()
        check(L.gbpx_bp_create(int(discard_static_vs_kinematic), int(discard_kinematic_vs_kinematic), ctypes.byref(h)),
              "gbpx_bp_create")
        self._h = h
        self._L = L

    def release(self):
        if self._h:
            self._L.gbpx_bp_release(self._h)
            self._h = None

    __del__ = release

    def update(self, created, updated, removed, bounds, groups, distances, capacity):
        c = np.ascontiguousarray(created if created is not None else [], dtype=np.uint32)
        u = np.ascontiguousarray(updated if updated is not None else [], dtype=np.uint32)
        r = np.ascontiguousarray(removed if removed is not None else [], dtype=np.uint32)
        b = np.ascontiguousarray(bounds, dtype=np.float32)
        g = np.ascontiguousarray(groups, dtype=np.uint32)
        d = np.ascontiguousarray(distances, dtype=np.float32)
        check(self._L.gbpx_bp_update(self._h, _ptr(c), len(c), _ptr(u), len(u), _ptr(r), len(r), _ptr(b), _ptr(g), _ptr(d),
                                     int(capacity)), "PxBroadPhase::update")

    def fetch_results(self):
        """Returns (created, lost) as (n, 2) uint32 arrays of handles, id0 < id1, sorted."""
        cp, lp = _u32p(), _u32p()
        nc, nl = ctypes.c_uint32(), ctypes.c_uint32()
        check(self._L.gbpx_bp_fetch_results(self._h, ctypes.byref(cp), ctypes.byref(nc), ctypes.byref(lp), ctypes.byref(nl)),
              "PxBroadPhase::fetchResults")
        created = np.ctypeslib.as_array(cp, shape=(nc.value * 2,)).reshape(-1, 2).copy() if nc.value else np.zeros((0, 2), np.uint32)
        lost = np.ctypeslib.as_array(lp, shape=(nl.value * 2,)).reshape(-1, 2).copy() if nl.value else np.zeros((0, 2), np.uint32)
        return created, lost

    def set_sweep(self, tiled):
        """Sweep kernels for the following updates: True = shared-memory tiled (default),
        False = one warp per updated box / one thread per other box (same pairs)."""
        self._L.gbpx_bp_set_sweep.argtypes = [ctypes.c_void_p, ctypes.c_int]
        check(self._L.gbpx_bp_set_sweep(self._h, 1 if tiled else 0), "gbpx_bp_set_sweep")

    def timing(self):
        """(host ms staging the user's arrays, device ms) of the last update + fetch."""
        out = np.zeros(2, np.float32)
        self._L.gbpx_bp_timing.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        check(self._L.gbpx_bp_timing(self._h, _ptr(out)), "gbpx_bp_timing")
        return float(out[0]), float(out[1])

    def stats(self):
        out = np.zeros(4, np.uint64)
        check(self._L.gbpx_bp_stats(self._h, _ptr(out)), "gbpx_bp_stats")
        return {"live": int(out[0]), "updated": int(out[1]), "found": int(out[2]), "active": int(out[3])}
