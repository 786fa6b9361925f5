"""Generates the golden fixtures in tests/golden/ by running the REFERENCE
(PhysX built from its own sources by oracle/ref/Makefile into
oracle/_ref/libpxref.so) on seeded synthetic inputs.

Run on the development machine, where the reference sources exist:

    make -C oracle/ref -j8 && python tests/golden/make_golden.py

Each fixture stores its inputs and the reference's outputs, so the tests on
machines without the reference need neither the reference nor this script.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle_libs import CpuBroadPhase, reference, run_contacts  # noqa: E402
from scenarios import bp_frames, np_pairs  # noqa: E402

BP_CASES = [
    # name, seed, boxes, frames, extent
    ("bp_dense", 11, 600, 5, 12.0),
    ("bp_sparse", 12, 1000, 4, 60.0),
]


def make_bp():
    for name, seed, n, frames, extent in BP_CASES:
        ref = CpuBroadPhase("pxref")
        out = {}
        for f, fr in enumerate(bp_frames(seed, n, frames, extent=extent)):
            created, lost = ref.update(fr)
            for k in ("created", "updated", "removed", "bounds", "groups", "distances"):
                out["f%d_%s" % (f, k)] = fr[k]
            out["f%d_capacity" % f] = np.array(fr["capacity"])
            out["f%d_ref_created" % f] = created
            out["f%d_ref_lost" % f] = lost
        out["frames"] = np.array(frames)
        ref.release()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)


NP_CASES = [
    # name, seed, pairs: near-contact pairs of every sphere/plane/capsule/box combination
    ("np_mixed", 17, 3000),
]


def make_np():
    for name, seed, n in NP_CASES:
        pairs = np_pairs(seed, n)
        cnt, out = run_contacts("pxref", pairs, max_per_pair=8)
        packed = np.concatenate([out[i, :cnt[i]] for i in range(n) if cnt[i]]) if cnt.sum() else np.zeros((0, 8), np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), counts=cnt, contacts=packed.astype(np.float32),
                            contact_distance=np.float32(0.04), tolerance_length=np.float32(1.0), **pairs)
        print("wrote", name)


if __name__ == "__main__":
    if reference() is None:
        sys.exit("oracle/_ref/libpxref.so is missing: build it with make -C oracle/ref")
    which = sys.argv[1:] or ["bp", "np"]
    if "bp" in which:
        make_bp()
    if "np" in which:
        make_np()
