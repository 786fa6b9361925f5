"""One large scene: the reference immediate-mode frame (ABP broadphase,
PxGenerateContacts, PxBatchConstraintsTGS, TGS solve and integrate, pair caches
and friction patches kept between frames) over one scene of any size, every
stage spread over the whole GPU.  The batched world gives each scene one warp
or one block and holds at most 65,535 bodies per scene; this class is for single
scenes of tens of thousands of bodies and more.
"""
import ctypes

import numpy as np

from . import check, lib
from .world import DEFAULT_PARAMS, param_vector

_p = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

STAGES = ("bounds + broadphase", "narrowphase", "constraints + batching", "bodies + rows", "iterations", "write-back")


def _setup():
    L = lib()
    if not getattr(L, "_scene_ready", False):
        L.gbpx_scene_create.argtypes = [ctypes.c_uint32] + [ctypes.c_void_p] * 4 + [ctypes.c_uint32] + [ctypes.c_void_p] * 5 + \
            [ctypes.POINTER(ctypes.c_void_p)]
        L.gbpx_scene_release.argtypes = [ctypes.c_void_p]
        L.gbpx_scene_release.restype = None
        L.gbpx_scene_step.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.gbpx_scene_get_bodies.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_scene_set_bodies.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_scene_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_scene_time_steps.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        L.gbpx_scene_step_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
        L._scene_ready = True
    return L


class Scene:
    """One scene resident on the GPU.  `scene` is a dict with one scene's arrays
    (rigid, types, geoms, friction, static_poses, static_types, static_geoms), as
    physx_gb300.workloads builds them."""

    def __init__(self, scene, params=None, persistent=None):
        L = _setup()
        p = dict(DEFAULT_PARAMS)
        p.update(params or {})
        if persistent is not None:
            p["persistent"] = bool(persistent)
        pv, it = param_vector(p)
        self._keep = [np.ascontiguousarray(scene["rigid"]), np.ascontiguousarray(scene["types"], np.int32),
                      np.ascontiguousarray(scene["geoms"], np.float32), np.ascontiguousarray(scene["friction"], np.float32),
                      np.ascontiguousarray(scene["static_poses"], np.float32), np.ascontiguousarray(scene["static_types"], np.int32),
                      np.ascontiguousarray(scene["static_geoms"], np.float32), pv, it]
        k = self._keep
        h = ctypes.c_void_p()
        check(L.gbpx_scene_create(len(k[0]), _p(k[0]), _p(k[1]), _p(k[2]), _p(k[3]), len(k[4]), _p(k[4]), _p(k[5]), _p(k[6]), _p(pv), _p(it),
                                  ctypes.byref(h)), "gbpx_scene_create")
        self._h, self._L = h, L
        self.nb_bodies = len(k[0])
        self.rigid_dtype = k[0].dtype

    def release(self):
        if getattr(self, "_h", None):
            self._L.gbpx_scene_release(self._h)
            self._h = None

    __del__ = release

    def step(self, n=1):
        check(self._L.gbpx_scene_step(self._h, n), "gbpx_scene_step")

    def get_bodies(self, out=None):
        out = np.empty(self.nb_bodies, self.rigid_dtype) if out is None else out
        check(self._L.gbpx_scene_get_bodies(self._h, _p(out)), "gbpx_scene_get_bodies")
        return out

    def set_bodies(self, rigid):
        rigid = np.ascontiguousarray(rigid)
        check(self._L.gbpx_scene_set_bodies(self._h, _p(rigid)), "gbpx_scene_set_bodies")

    def stats(self):
        out = np.zeros(4, np.uint64)
        check(self._L.gbpx_scene_stats(self._h, _p(out)), "gbpx_scene_stats")
        return dict(pairs=int(out[0]), constraints=int(out[1]), contacts=int(out[2]), partitions=int(out[3]))

    def set_device_batching(self, enable=True):
        """PxBatchConstraintsTGS's rule on the device (default) or on the host; the
        results are the same."""
        self._L.gbpx_scene_set_device_batching.argtypes = [ctypes.c_void_p, ctypes.c_int]
        check(self._L.gbpx_scene_set_device_batching(self._h, int(bool(enable))), "gbpx_scene_set_device_batching")

    def batch_info(self):
        """(colouring passes, batched on the device) of the last frame."""
        out = np.zeros(2, np.uint32)
        self._L.gbpx_scene_batch_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        check(self._L.gbpx_scene_batch_info(self._h, _p(out)), "gbpx_scene_batch_info")
        return int(out[0]), bool(out[1])

    def time_steps(self, n):
        """Runs n frames; returns (ms per frame, {stage: ms per frame}) from CUDA events on the scene's stream."""
        out = np.zeros(1 + len(STAGES), np.float32)
        check(self._L.gbpx_scene_time_steps(self._h, n, _p(out)), "gbpx_scene_time_steps")
        return float(out[0]), dict(zip(STAGES, (float(x) for x in out[1:])))

    def step_host(self, rigid_in, rigid_out, n=1):
        """Bodies in from host memory, n frames, bodies out; returns event-timed milliseconds."""
        ms = ctypes.c_float(0)
        check(self._L.gbpx_scene_step_host(self._h, _p(rigid_in), _p(rigid_out), n, ctypes.byref(ms)), "gbpx_scene_step_host")
        return ms.value
