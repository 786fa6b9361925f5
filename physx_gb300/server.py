"""Serving pool: scenes resident in HBM, requests "advance scene k by n steps"
served by continuous batching (libgbpx gbpx_server_*)."""
import ctypes

import numpy as np

from . import check, lib
from .world import DEFAULT_PARAMS, param_vector

_p = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def _setup():
    L = lib()
    if not getattr(L, "_server_ready", False):
        L.gbpx_server_create.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
        L.gbpx_server_run_load.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32] + [ctypes.c_void_p] * 9
        L.gbpx_server_release.argtypes = [ctypes.c_void_p]
        L.gbpx_server_slot_bytes.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        L.gbpx_server_slot_bytes.restype = ctypes.c_uint64
        L.gbpx_server_admit.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 4 + [ctypes.c_uint32] + [ctypes.c_void_p] * 3 + \
            [ctypes.POINTER(ctypes.c_uint32)]
        L.gbpx_server_retire.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.gbpx_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double]
        L.gbpx_server_pump.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]
        L.gbpx_server_clock.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        L.gbpx_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        L.gbpx_server_read_scene.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        L.gbpx_server_snapshot_scene.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                                                 ctypes.POINTER(ctypes.c_uint64)]
        L.gbpx_server_restore_scene.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32)]
        L.gbpx_server_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L._server_ready = True
    return L


def slot_bytes(capacity, statics=1, pairs_per_body=8, persistent=True):
    return int(_setup().gbpx_server_slot_bytes(capacity, statics, pairs_per_body, int(bool(persistent))))


def slots_for_budget(capacities, budget_bytes, weights=None, statics=1, pairs_per_body=8, persistent=True):
    """Slots per class so that the pool fits `budget_bytes`; `weights` is the expected
    share of scenes per class (equal by default, the log-uniform body-count case)."""
    w = np.ones(len(capacities)) if weights is None else np.asarray(weights, np.float64)
    w = w / w.sum()
    per = sum(wi * slot_bytes(c, statics, pairs_per_body, persistent) for wi, c in zip(w, capacities))
    total = int(budget_bytes // per)
    return [max(1, int(total * wi)) for wi in w]


class Server:
    _h = None

    def __init__(self, capacities, slots, statics=1, pairs_per_body=8, lanes_per_class=1, **params):
        L = _setup()
        p = dict(DEFAULT_PARAMS)
        p.update(params)
        pv, it = param_vector(p)
        cap = np.ascontiguousarray(capacities, np.uint32)
        sl = np.ascontiguousarray(slots, np.uint32)
        h = ctypes.c_void_p()
        check(L.gbpx_server_create(len(cap), _p(cap), _p(sl), statics, _p(pv), _p(it), pairs_per_body, lanes_per_class, ctypes.byref(h)),
              "gbpx_server_create")
        self._h, self._L = h, L
        self._sizes = {}
        self._dtype = None

    def release(self):
        if self._h:
            self._L.gbpx_server_release(self._h)
            self._h = None

    __del__ = release

    def admit(self, scene):
        """scene: one scene in the world layout (rigid, types, geoms, friction, static_poses, static_types, static_geoms)."""
        rb = np.ascontiguousarray(scene["rigid"])
        k = [np.ascontiguousarray(scene["types"], np.int32), np.ascontiguousarray(scene["geoms"], np.float32),
             np.ascontiguousarray(scene["friction"], np.float32), np.ascontiguousarray(scene["static_poses"], np.float32),
             np.ascontiguousarray(scene["static_types"], np.int32), np.ascontiguousarray(scene["static_geoms"], np.float32)]
        out = ctypes.c_uint32()
        check(self._L.gbpx_server_admit(self._h, len(rb), _p(rb), _p(k[0]), _p(k[1]), _p(k[2]), len(k[3]), _p(k[3]), _p(k[4]), _p(k[5]),
                                        ctypes.byref(out)), "gbpx_server_admit")
        self._sizes[out.value] = len(rb)
        self._dtype = rb.dtype
        return out.value

    def retire(self, scene):
        check(self._L.gbpx_server_retire(self._h, scene), "gbpx_server_retire")

    def submit(self, scene, steps, tag, arrival=-1.0):
        check(self._L.gbpx_server_submit(self._h, scene, steps, tag, arrival), "gbpx_server_submit")

    def pump(self):
        n = ctypes.c_uint32()
        check(self._L.gbpx_server_pump(self._h, ctypes.byref(n)), "gbpx_server_pump")
        return n.value

    def clock(self):
        t = ctypes.c_double()
        check(self._L.gbpx_server_clock(self._h, ctypes.byref(t)), "gbpx_server_clock")
        return t.value

    def poll(self, capacity=65536):
        tags = np.zeros(capacity, np.uint64)
        lat = np.zeros(capacity, np.float64)
        n = ctypes.c_uint32()
        check(self._L.gbpx_server_poll(self._h, _p(tags), _p(lat), capacity, ctypes.byref(n)), "gbpx_server_poll")
        return tags[:n.value].copy(), lat[:n.value].copy()

    def read_scene(self, scene):
        out = np.zeros(self._sizes[scene], self._dtype)
        check(self._L.gbpx_server_read_scene(self._h, scene, _p(out)), "gbpx_server_read_scene")
        return out

    def snapshot(self, scene):
        """The scene's state between steps (bytes): bodies, shapes, statics and its
        pair list with contact manifolds and friction patches."""
        n = ctypes.c_uint64(0)
        check(self._L.gbpx_server_snapshot_scene(self._h, scene, None, 0, ctypes.byref(n)), "gbpx_server_snapshot_scene")
        out = np.zeros(n.value, np.uint8)
        check(self._L.gbpx_server_snapshot_scene(self._h, scene, _p(out), n.value, ctypes.byref(n)), "gbpx_server_snapshot_scene")
        return out

    def restore(self, snap):
        """Admits a snapshot as a new scene; returns its id."""
        snap = np.ascontiguousarray(snap, np.uint8)
        sid = ctypes.c_uint32(0)
        check(self._L.gbpx_server_restore_scene(self._h, _p(snap), len(snap), ctypes.byref(sid)), "gbpx_server_restore_scene")
        self._sizes[sid.value] = int(np.frombuffer(snap[8:12].tobytes(), np.uint32)[0])
        return sid.value

    def stats(self):
        out = np.zeros(4, np.uint64)
        check(self._L.gbpx_server_stats(self._h, _p(out)), "gbpx_server_stats")
        return dict(body_steps=int(out[0]), steps=int(out[1]), live=int(out[2]), inflight=int(out[3]))

    def drain(self, timeout=60.0):
        """Pumps until every submitted request has completed; returns (tags, latencies)."""
        import time
        tags, lats = [], []
        t_end = time.time() + timeout
        while time.time() < t_end:
            self.pump()
            t, l_ = self.poll()
            tags.append(t)
            lats.append(l_)
            st = self.stats()
            if st["inflight"] == 0 and self.pump() == 0 and self.stats()["inflight"] == 0:
                t, l_ = self.poll()
                tags.append(t)
                lats.append(l_)
                break
        return np.concatenate(tags), np.concatenate(lats)

    def run_load(self, library, seconds, rate, steps=(1, 8), life=(500, 5000), seed=5):
        """The open-loop Poisson load run in the library (gbpx_server_run_load) over a
        library of scenes (dicts with one static shape each); returns its figures."""
        off = np.zeros(len(library) + 1, np.uint32)
        off[1:] = np.cumsum([len(sc["rigid"]) for sc in library])
        cat = lambda k, dt: np.ascontiguousarray(np.concatenate([np.asarray(sc[k]).reshape(len(sc[k]), -1) for sc in library]), dt)  # noqa: E731
        rigid = np.ascontiguousarray(np.concatenate([sc["rigid"] for sc in library]))
        types, geoms, fr = cat("types", np.int32), cat("geoms", np.float32), cat("friction", np.float32)
        spose, stype, sgeom = cat("static_poses", np.float32), cat("static_types", np.int32), cat("static_geoms", np.float32)
        out = np.zeros(16, np.float64)
        check(self._L.gbpx_server_run_load(self._h, float(seconds), float(rate), int(steps[0]), int(steps[1]), int(life[0]), int(life[1]),
                                           int(seed), len(library), _p(off), _p(rigid), _p(types), _p(geoms), _p(fr), _p(spose), _p(stype),
                                           _p(sgeom), _p(out)), "gbpx_server_run_load")
        keys = ("seconds", "submitted", "completed", "body_steps", "p50_ms", "p99_ms", "p50_ms_512", "p99_ms_512", "p50_ms_per_step_512",
                "p99_ms_per_step_512", "live_scenes", "retired", "admitted_after_start", "lane_steps", "lanes")
        return {k: float(v) for k, v in zip(keys, out)}
