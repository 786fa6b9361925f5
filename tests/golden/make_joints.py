"""Golden fixtures for the joint path: seeded joint scenes (tests/joint_scenes.py)
stepped through the reference built from source (oracle/_ref/libpxref.so,
harness pxref_joint_frame: PxBatchConstraintsTGS, PxCreateJointConstraintsTGS,
PxSolveConstraintsTGS, PxIntegrateSolverBodiesTGS), each frame's rows written
from the poses the previous frame left.  Sampled frames keep their inputs
(bodies, rows, parameters) and the reference's outputs.

    python tests/golden/make_joints.py      (development machine, after make -C oracle/ref)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from joint_scenes import joint_frame, make_joint_scene     # noqa: E402
from oracle_libs import advance_rigid, reference, run_joints  # noqa: E402

CASES = {
    # name: (seed, chains, links, frames run, frames kept)
    "joints_chains": (11, 6, (3, 8), 90, (0, 1, 2, 45, 89)),
    "joints_large": (12, 40, (2, 9), 40, (0, 20, 39)),
}


def main():
    if reference() is None:
        raise SystemExit("reference library not built (make -C oracle/ref)")
    for name, (seed, chains, links, frames, keep) in CASES.items():
        sc = make_joint_scene(seed, nb_chains=chains, links=links)
        rigid = sc["rigid"]
        out = {}
        for f in range(frames):
            fr = joint_frame(sc, rigid)
            r = run_joints("pxref", fr)
            if f in keep:
                p = "f%d_" % f
                out[p + "rigid"] = rigid.view(np.uint8).reshape(len(rigid), -1).copy()
                out[p + "rows"] = fr["rows"].view(np.uint8).reshape(len(fr["rows"]), -1).copy()
                out[p + "row_start"], out[p + "row_count"], out[p + "params"] = fr["row_start"], fr["row_count"], fr["params"]
                for k, v in r.items():
                    out[p + "ref_" + k] = v
            rigid = advance_rigid(rigid, r["vel"], r["pose"])
        A = np.array([j["a"] for j in sc["joints"]], np.uint32)
        B = np.array([j["b"] for j in sc["joints"]], np.uint32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=np.array(keep, np.int32), joint_a=A, joint_b=B,
                            static_poses=sc["static_poses"], nb_dyn=np.int32(sc["nb_dyn"]), **out)
        types = np.concatenate([out["f%d_ref_header_type" % f] for f in keep])
        print(name, "bodies", sc["nb_dyn"], "joints", len(A), "header types", np.bincount(types).tolist(),
              "broken", int(sum(out["f%d_ref_broken" % f].sum() for f in keep)))


if __name__ == "__main__":
    main()
