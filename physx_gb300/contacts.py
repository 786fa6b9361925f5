"""immediate::PxGenerateContacts mirror over the GB300 narrowphase.

Mirrors physx/include/PxImmediateMode.h:267 for sphere / plane / capsule / box
and convex-core (PxConvexCoreGeometry) geometries with a fresh PxCache per
pair.  Pairs are given as arrays: type0/type1 (PxGeometryType; a convex core is
4 | its PxConvexCore::Type << 8, see workloads.convex_core_type), geom0/geom1
(4 floats; a convex core's core floats and its margin last), pose0/pose1
(7 floats qx qy qz qw px py pz).  Contacts come back as
(counts, contacts[n, max, 8]).
"""
import ctypes

import numpy as np

from . import GbpxError, check, lib

_ARG_KEYS = ("type0", "geom0", "type1", "geom1", "pose0", "pose1")
_DTYPES = (np.int32, np.float32, np.int32, np.float32, np.float32, np.float32)


def _setup():
    L = lib()
    if not getattr(L, "_np_ready", False):
        L.gbpx_generate_contacts.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                                                     ctypes.c_float, ctypes.c_void_p, ctypes.c_uint32,
                                                                     ctypes.c_void_p]
        L._np_ready = True
    return L


def generate_contacts(pairs, contact_distance=0.04, mesh_contact_margin=0.01, tolerance_length=1.0, max_per_pair=4):
    L = _setup()
    arrs = [np.ascontiguousarray(pairs[k], dtype=d) for k, d in zip(_ARG_KEYS, _DTYPES)]
    n = len(arrs[0])
    out = np.zeros((n, max_per_pair, 8), np.float32)
    cnt = np.zeros(n, np.uint32)
    rc = L.gbpx_generate_contacts(*[a.ctypes.data_as(ctypes.c_void_p) for a in arrs], n, contact_distance, mesh_contact_margin,
                                  tolerance_length, out.ctypes.data_as(ctypes.c_void_p), max_per_pair,
                                  cnt.ctypes.data_as(ctypes.c_void_p))
    if rc not in (0, -3):
        check(rc, "PxGenerateContacts")
    if rc == -3:
        raise GbpxError(rc, "PxGenerateContacts (more contacts than max_per_pair)")
    return cnt, out


MANIFOLD_BYTES = 288


class CachedContacts:
    """PxGenerateContacts over the same pairs frame after frame with persistent
    caches: each pair's contact manifold (plane-capsule, plane-box, capsule-box and
    box-box keep one, as PxCache does) is carried from one call to the next in a
    288-byte record per pair held here."""

    def __init__(self, nb_pairs):
        L = _setup()
        if not getattr(L, "_np_cached_ready", False):
            L.gbpx_generate_contacts_cached.argtypes = ([ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                                                                  ctypes.c_float, ctypes.c_void_p, ctypes.c_uint32,
                                                                                  ctypes.c_void_p, ctypes.c_void_p])
            L._np_cached_ready = True
        self.L = L
        self.state = np.zeros(nb_pairs * MANIFOLD_BYTES, np.uint8)

    def reset(self):
        """Fresh caches for every pair."""
        self.state[:] = 0

    def run(self, pairs, contact_distance=0.04, mesh_contact_margin=0.01, tolerance_length=1.0, max_per_pair=4):
        arrs = [np.ascontiguousarray(pairs[k], dtype=d) for k, d in zip(_ARG_KEYS, _DTYPES)]
        n = len(arrs[0])
        if n * MANIFOLD_BYTES != len(self.state):
            raise ValueError("pair count differs from the cache count")
        out = np.zeros((n, max_per_pair, 8), np.float32)
        cnt = np.zeros(n, np.uint32)
        rc = self.L.gbpx_generate_contacts_cached(*[a.ctypes.data_as(ctypes.c_void_p) for a in arrs], n, contact_distance,
                                                  mesh_contact_margin, tolerance_length, out.ctypes.data_as(ctypes.c_void_p),
                                                  max_per_pair, cnt.ctypes.data_as(ctypes.c_void_p),
                                                  self.state.ctypes.data_as(ctypes.c_void_p))
        if rc == -3:
            raise GbpxError(rc, "PxGenerateContacts (more contacts than max_per_pair)")
        check(rc, "PxGenerateContacts")
        return cnt, out
