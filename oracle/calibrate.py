"""Times the oracle restatement (oracle/liboracle.so) against the reference
built from its own sources (oracle/_ref/libpxref.so) on the same inputs, one
host thread each, so that speed-ups quoted against the restatement can be
converted to speed-ups against the reference.  Test infrastructure: run on the
development machine, where the reference build exists.

    python oracle/calibrate.py            # prints one JSON line

Workloads: the 210-box pyramid (300 persistent steps), the 1M-box broadphase
(one update frame of 10 % moved boxes after the creating frame), and a
256-scene sample of the 4096-scene batched workload (40 persistent steps of
pre-roll, then 5 timed persistent steps).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle_libs import CpuBroadPhase, PersistentScenes, reference  # noqa: E402
from scenarios import bp_frames  # noqa: E402
from physx_gb300.workloads import batched_scenes, pyramid_scene  # noqa: E402
from physx_gb300.world import DEFAULT_PARAMS  # noqa: E402


def time_pyramid(which, steps=300):
    ps = PersistentScenes(which, pyramid_scene(), DEFAULT_PARAMS)
    t = time.perf_counter()
    ps.step(steps)
    dt = time.perf_counter() - t
    ps.release()
    return dt


def time_broadphase(which, n=1_000_000):
    import numpy as np
    bp = CpuBroadPhase(which)
    dt = 0.0
    for f, fr in enumerate(bp_frames(3, n, 2, extent=1000.0, move_frac=0.1, edge_cases=False, removals=False, distances=False)):
        fr["groups"] = ((np.arange(n, dtype=np.uint32) + 1) << 3) | 2
        t = time.perf_counter()
        bp.update(fr)
        if f:
            dt += time.perf_counter() - t
    bp.release()
    return dt


def time_batched(which, nb=256, preroll=40, steps=5):
    import numpy as np
    sys.path.insert(0, ROOT)
    from bench import cpu_sample, split_scenes
    scenes = batched_scenes(4, 4096)
    sample = split_scenes(scenes, cpu_sample(4096, nb))
    ps = PersistentScenes(which, sample, DEFAULT_PARAMS)
    ps.step(preroll)
    t = time.perf_counter()
    ps.step(steps)
    dt = time.perf_counter() - t
    ps.release()
    return dt


if __name__ == "__main__":
    if reference() is None:
        sys.exit("the reference build (oracle/_ref/libpxref.so) is missing: make -C oracle/ref")
    out = {}
    for name, fn in (("pyramid_300_steps", time_pyramid), ("broadphase_1m_frame", time_broadphase), ("batched_256_scenes_5_steps", time_batched)):
        ref, orc = fn("pxref"), fn("orc")
        out[name] = dict(reference_s=ref, restatement_s=orc, restatement_over_reference=orc / ref)
    out["host"] = os.uname().machine
    print(json.dumps(out))
