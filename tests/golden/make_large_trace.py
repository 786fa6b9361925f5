"""Writes tests/golden/large_scene_trace.npz: physical statistics of the
single-large-scene workload (100k sphere / box / capsule bodies dropped onto a
plane, the snippet's persistent frame: ABP, PxGenerateContacts with caches,
PxBatchConstraintsTGS, TGS 4/1 with friction data kept) over 600 steps, run by
the REFERENCE (oracle/_ref/libpxref.so, built from the reference's sources by
oracle/ref/Makefile) on one host thread.  Per step: kinetic energy, ground
clearance of the lowest body, mean and top height, resting fraction.

    make -C oracle/ref -j8 && python tests/golden/make_large_trace.py [steps]

The run takes tens of minutes (one thread, 100k bodies); the GPU test only reads
the statistics.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle_libs import PersistentScenes, reference  # noqa: E402
from trace_stats import FIELDS, body_checksum, step_stats  # noqa: E402
from physx_gb300.workloads import as_world, large_scene  # noqa: E402
from physx_gb300.world import DEFAULT_PARAMS  # noqa: E402

if __name__ == "__main__":
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 600
    which = sys.argv[2] if len(sys.argv) > 2 else "pxref"
    if which == "pxref" and reference() is None:
        sys.exit("the reference build (oracle/_ref/libpxref.so) is missing")
    sc = large_scene()
    ps = PersistentScenes(which, as_world(sc), DEFAULT_PARAMS)
    rows = []
    t = time.time()
    for s in range(steps):
        rb = ps.step(1)
        rows.append([step_stats(rb, sc["types"], sc["geoms"])[f] for f in FIELDS])
        if s % 50 == 0:
            print("step", s, rows[-1], "%.0f s" % (time.time() - t), flush=True)
    ps.release()
    out = os.path.join(HERE, "large_scene_trace.npz" if which == "pxref" else "large_scene_trace_%s.npz" % which)
    np.savez_compressed(out, stats=np.array(rows, np.float64), fields=np.array(FIELDS), checksum=np.array(body_checksum(sc["rigid"]), np.uint64),
                        steps=np.array(steps))
    print("wrote", out)
