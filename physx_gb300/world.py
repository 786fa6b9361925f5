"""Batched multi-scene world: thousands of independent scenes stepped by one
CUDA graph per step (warp-per-scene or block-per-scene stage kernels, picked by
scene size; autotune() chooses the threshold for the scene-size histogram), all
state resident in HBM.  Each scene's frame is the reference immediate-mode loop
(ABP broadphase, PxGenerateContacts, TGS) with the snippet's persistent pair
state (contact manifolds and friction patches kept between steps) by default.
"""
import ctypes

import numpy as np

from . import check, lib

_p = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

DEFAULT_PARAMS = dict(dt=1.0 / 60.0, gravity=(0.0, -9.81, 0.0), contact_distance=0.04, tolerance_length=1.0, bounds_margin=0.02,
                      bounce_threshold=-2.0, friction_offset_threshold=0.04, correlation_distance=0.025, static_friction=0.5,
                      nb_pos=4, nb_vel=1, persistent=True)


def param_vector(p):
    g = p["gravity"]
    params = np.array([p["dt"], g[0], g[1], g[2], p["contact_distance"], p["tolerance_length"], p["bounds_margin"],
                       p["bounce_threshold"], p["friction_offset_threshold"], p["correlation_distance"], p["static_friction"],
                       1.0 if p.get("persistent", True) else 0.0], np.float32)
    return params, np.array([p["nb_pos"], p["nb_vel"]], np.uint32)


def _setup():
    L = lib()
    if not getattr(L, "_world_ready", False):
        L.gbpx_world_create.argtypes = [ctypes.c_uint32] + [ctypes.c_void_p] * 11 + [ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
        L.gbpx_world_release.argtypes = [ctypes.c_void_p]
        L.gbpx_world_step.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int]
        L.gbpx_world_synchronize.argtypes = [ctypes.c_void_p]
        L.gbpx_world_get_bodies.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_set_bodies.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_status.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_scene_pairs.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                             ctypes.POINTER(ctypes.c_uint32)]
        L.gbpx_world_time_steps.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.gbpx_world_time_plain.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]
        L.gbpx_world_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_kind_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_world_set_large_bodies.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.gbpx_world_autotune.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                                          ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float)]
        L.gbpx_world_set_solve_variant.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.gbpx_world_time_stages.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        L.gbpx_world_step_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_float)]
        L.gbpx_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
        L.gbpx_host_free.argtypes = [ctypes.c_void_p]
        L._world_ready = True
    return L


class World:
    """`scenes` dict: body_count (S,), static_count (S,), rigid (PxRigidBodyData records),
    types (N,), geoms (N,4), friction (N,), static_poses (M,7), static_types (M,), static_geoms (M,4)."""

    _h = None

    def __init__(self, scenes, pairs_per_body=8, **params):
        L = _setup()
        p = dict(DEFAULT_PARAMS)
        p.update(params)
        self.params = p
        pv, it = param_vector(p)
        self._keep = [np.ascontiguousarray(scenes["body_count"], np.uint32), np.ascontiguousarray(scenes["static_count"], np.uint32),
                      np.ascontiguousarray(scenes["rigid"]), np.ascontiguousarray(scenes["types"], np.int32),
                      np.ascontiguousarray(scenes["geoms"], np.float32), np.ascontiguousarray(scenes["friction"], np.float32),
                      np.ascontiguousarray(scenes["static_poses"], np.float32), np.ascontiguousarray(scenes["static_types"], np.int32),
                      np.ascontiguousarray(scenes["static_geoms"], np.float32), pv, it]
        h = ctypes.c_void_p()
        k = self._keep
        check(L.gbpx_world_create(len(k[0]), _p(k[0]), _p(k[1]), _p(k[2]), _p(k[3]), _p(k[4]), _p(k[5]), _p(k[6]), _p(k[7]), _p(k[8]),
                                  _p(pv), _p(it), pairs_per_body, ctypes.byref(h)), "gbpx_world_create")
        self._h, self._L = h, L
        self.pairs_per_body = pairs_per_body
        self.nb_bodies = len(k[2])
        self.rigid_dtype = k[2].dtype

    def step_checked(self, n=1, max_pairs_per_body=128):
        """n steps, one at a time; a step after which a scene reports that its pair
        slots overflowed (status bit 1) is taken again, from the bodies before it, in
        a world with twice the pair slots per body (pair history restarts there),
        until it fits or max_pairs_per_body is reached (then GbpxError).  Returns the
        pair slots per body in use."""
        from . import GbpxError
        for _ in range(n):
            before = self.get_bodies()
            self.step(1, graph=False)
            while (self.status() & 1).any():
                if self.pairs_per_body * 2 > max_pairs_per_body:
                    raise GbpxError(-3, "World.step_checked: pair slots")
                k = self._keep
                h = ctypes.c_void_p()
                check(self._L.gbpx_world_create(len(k[0]), _p(k[0]), _p(k[1]), _p(before), _p(k[3]), _p(k[4]), _p(k[5]), _p(k[6]),
                                                _p(k[7]), _p(k[8]), _p(k[9]), _p(k[10]), self.pairs_per_body * 2, ctypes.byref(h)),
                      "gbpx_world_create")
                self._L.gbpx_world_release(self._h)
                self._h = h
                self.pairs_per_body *= 2
                self.step(1, graph=False)
        return self.pairs_per_body

    def release(self):
        if self._h:
            self._L.gbpx_world_release(self._h)
            self._h = None
        for ptr in getattr(self, "_pinned", []):
            self._L.gbpx_host_free(ptr)
        self._pinned = []

    __del__ = release

    def step(self, n=1, graph=True):
        check(self._L.gbpx_world_step(self._h, n, int(graph)), "gbpx_world_step")

    def synchronize(self):
        check(self._L.gbpx_world_synchronize(self._h), "gbpx_world_synchronize")

    def get_bodies(self, out=None):
        out = np.empty(self.nb_bodies, self.rigid_dtype) if out is None else out
        check(self._L.gbpx_world_get_bodies(self._h, _p(out)), "gbpx_world_get_bodies")
        return out

    def set_bodies(self, rigid):
        rigid = np.ascontiguousarray(rigid)
        check(self._L.gbpx_world_set_bodies(self._h, _p(rigid)), "gbpx_world_set_bodies")

    def status(self):
        st = np.zeros(len(self._keep[0]), np.uint32)
        check(self._L.gbpx_world_status(self._h, _p(st)), "gbpx_world_status")
        return st

    def info(self):
        out = np.zeros(8, np.uint64)
        check(self._L.gbpx_world_info(self._h, _p(out)), "gbpx_world_info")
        return dict(scenes=int(out[0]), bodies=int(out[1]), statics=int(out[2]), pair_slots=int(out[3]), grid_blocks=int(out[4]),
                    device_bytes=int(out[5]), kernels_per_step=int(out[6]), large_bodies=int(out[7]))

    def time_steps(self, n, graph=True):
        """Milliseconds for n device-resident steps (CUDA events on the world stream)."""
        ms = ctypes.c_float(0)
        check(self._L.gbpx_world_time_steps(self._h, n, int(graph), ctypes.byref(ms)), "gbpx_world_time_steps")
        return ms.value

    def time_plain(self, first, count):
        """Milliseconds to step scenes [first, first+count) one scene per launch."""
        ms = ctypes.c_float(0)
        check(self._L.gbpx_world_time_plain(self._h, first, count, ctypes.byref(ms)), "gbpx_world_time_plain")
        return ms.value

    def stats(self):
        out = np.zeros(4, np.uint64)
        check(self._L.gbpx_world_stats(self._h, _p(out)), "gbpx_world_stats")
        return dict(pairs=int(out[0]), constraints=int(out[1]), contacts=int(out[2]), row_bytes=int(out[3]))

    def solve_profile(self):
        """Per scene after the last step: constraints, partitions, packed row bytes and the
        widest partition, as an (S, 4) uint32 array."""
        out = np.zeros((self.info()["scenes"], 4), np.uint32)
        check(self._L.gbpx_world_solve_profile(self._h, _p(out)), "gbpx_world_solve_profile")
        return out

    def set_large_bodies(self, n):
        """Scenes of more than n solver bodies run one block per scene in the scene
        stages (warp per scene below); results do not depend on it."""
        check(self._L.gbpx_world_set_large_bodies(self._h, int(n)), "gbpx_world_set_large_bodies")

    def autotune(self, sample_scenes=None, steps=3):
        """Picks the block-per-scene threshold for this world's scene-size histogram
        (timed on a temporary copy of a size-stratified sample of the scenes, all of
        them by default; cached per histogram), then the solve kernel and the
        preparation / heavy narrowphase blocks per SM; returns (threshold, ms per step
        of the sample with them, 0 if cached) and keeps the solve kernel in
        self.solve_variant (tuning() has the whole choice).  The sample should load the GPU like the whole
        world: warp-per-scene kernels need many scenes to fill it."""
        if sample_scenes is None:
            sample_scenes = len(self._keep[0])
        t = ctypes.c_uint32(0)
        v = ctypes.c_uint32(0)
        ms = ctypes.c_float(0)
        check(self._L.gbpx_world_autotune(self._h, sample_scenes, steps, ctypes.byref(t), ctypes.byref(v), ctypes.byref(ms)),
              "gbpx_world_autotune")
        self.solve_variant = v.value
        return t.value, ms.value

    def tuning(self):
        """{large_bodies, solve_variant, prep_blocks_per_sm, narrowphase_blocks_per_sm,
        resident_stream} in force (the autotuner's choice, or what was set by hand; 0
        blocks per SM = as many as fit)."""
        out = np.zeros(5, np.uint32)
        check(self._L.gbpx_world_tuning(self._h, _p(out)), "gbpx_world_tuning")
        return dict(large_bodies=int(out[0]), solve_variant=int(out[1]), prep_blocks_per_sm=int(out[2]),
                    narrowphase_blocks_per_sm=int(out[3]), resident_stream=int(out[4]))

    def set_resident_stream(self, levels):
        """Streamed rows in the resident solve (0-3, default 1): scenes filed above
        level `levels` go one level deeper, their rows streamed through a two-slot
        ring; results do not depend on it."""
        self._L.gbpx_world_set_resident_stream.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        check(self._L.gbpx_world_set_resident_stream(self._h, int(levels)), "gbpx_world_set_resident_stream")

    def set_occupancy(self, prep_blocks_per_sm=0, narrowphase_blocks_per_sm=0):
        """Persistent blocks per SM of the row preparation and of the capsule-box and
        box-box narrowphase kernels (0 = as many as fit); results do not depend on it."""
        self._L.gbpx_world_set_occupancy.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]
        check(self._L.gbpx_world_set_occupancy(self._h, int(prep_blocks_per_sm), int(narrowphase_blocks_per_sm)), "gbpx_world_set_occupancy")

    def set_solve_variant(self, v):
        """Solve kernel: 8 (default) the resident solve (each scene's rows and
        velocities on chip for all iterations); 0-7 the warp-per-scene solve, whose
        variants 0-2 keep velocities in shared memory with 0 / 256 / 512 B of row
        staging per lane, 3-5 the same with the velocities in HBM, 6 / 7 400 B with
        velocities on chip / in HBM.  Results do not depend on it."""
        check(self._L.gbpx_world_set_solve_variant(self._h, int(v)), "gbpx_world_set_solve_variant")

    def kind_counts(self):
        """Pairs of each pair kind in the last step, {narrowphase stage name: pairs}."""
        out = np.zeros(9, np.uint32)
        check(self._L.gbpx_world_kind_counts(self._h, _p(out)), "gbpx_world_kind_counts")
        return dict(zip(self.STAGES[1:10], (int(x) for x in out)))

    STAGES = ("broadphase", "np sphere-sphere", "np sphere-plane", "np sphere-capsule", "np sphere-box", "np plane-capsule",
              "np plane-box", "np capsule-capsule", "np capsule-box", "np box-box", "batching", "row preparation", "solve")

    def time_stages(self, n):
        """Average device milliseconds per kernel of a step, {stage name: ms} (un-captured steps)."""
        k = self.info()["kernels_per_step"]
        out = np.zeros(k, np.float32)
        check(self._L.gbpx_world_time_stages(self._h, n, _p(out)), "gbpx_world_time_stages")
        return dict(zip(self.STAGES, (float(x) for x in out)))

    def step_host(self, rigid_in, rigid_out, n=1, graph=True):
        """Upload bodies from host memory, step, download; returns event-timed milliseconds."""
        ms = ctypes.c_float(0)
        check(self._L.gbpx_world_step_host(self._h, _p(rigid_in), _p(rigid_out), n, int(graph), ctypes.byref(ms)), "gbpx_world_step_host")
        return ms.value

    def pinned_bodies(self):
        """A pinned host array of PxRigidBodyData records sized for this world."""
        ptr = ctypes.c_void_p()
        nbytes = self.nb_bodies * self.rigid_dtype.itemsize
        check(self._L.gbpx_host_alloc(nbytes, ctypes.byref(ptr)), "gbpx_host_alloc")
        buf = (ctypes.c_uint8 * nbytes).from_address(ptr.value)
        arr = np.frombuffer(buf, dtype=self.rigid_dtype, count=self.nb_bodies)
        self._pinned = getattr(self, "_pinned", []) + [ptr]
        return arr

    def scene_pairs(self, scene, capacity=1 << 16):
        keys = np.zeros(capacity, np.uint32)
        cnt = np.zeros(capacity, np.uint32)
        n = ctypes.c_uint32(0)
        check(self._L.gbpx_world_scene_pairs(self._h, scene, _p(keys), _p(cnt), capacity, ctypes.byref(n)), "gbpx_world_scene_pairs")
        m = min(n.value, capacity)
        return np.stack([keys[:m] >> 16, keys[:m] & 0xffff], 1), cnt[:m]
