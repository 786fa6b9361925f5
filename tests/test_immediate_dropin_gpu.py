"""libgbpx_immediate.so as a drop-in for the reference's immediate-mode TGS path:
tests/immediate_dropin.cpp is one frame written against the reference's
interface (PxGenerateContacts, PxConstructSolverBodiesTGS,
PxConstructStaticSolverBodyTGS, PxBatchConstraintsTGS,
PxCreateContactConstraintsTGS, PxSolveConstraintsTGS,
PxIntegrateSolverBodiesTGS) linked against this library; its result matches the
CPU oracle's frame on the same scene."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle_libs import run_tgs, scene_contacts, scene_pairs
from scenarios import random_scene
from test_oracle_golden import velocity_error

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp):
    exe = os.path.join(tmp, "immediate_dropin")
    lib_dir = os.path.join(ROOT, "physx_gb300")
    subprocess.check_call([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "immediate_dropin.cpp"), "-o", exe, "-L", lib_dir, "-lgbpx_immediate",
                           "-Wl,-rpath," + lib_dir])
    return exe


@pytest.mark.parametrize("shapes", [(0, 2), (0, 2, 3)])
def test_immediate_frame_matches_oracle(cuda_device, tmp_path, shapes):
    exe = _build(str(tmp_path))
    sc = random_scene(95, 30, shapes=shapes)
    A, B = scene_pairs(sc)
    n, m = len(sc["types"]), len(sc["static_poses"])
    fr = sc["friction"]
    pair_friction = np.array([(fr[a] + (fr[b] if b < n else 0.5)) * 0.5 for a, b in zip(A, B)], np.float32)
    params = np.array([1.0 / 60.0, 0.0, -9.81, 0.0, 0.04, 1.0, -2.0, 0.04, 0.025], np.float32)
    blob = b"".join([np.array([n, m, len(A)], np.uint32).tobytes(), np.ascontiguousarray(sc["rigid"]).tobytes(),
                     np.ascontiguousarray(sc["types"], np.int32).tobytes(), np.ascontiguousarray(sc["geoms"], np.float32).tobytes(),
                     np.ascontiguousarray(sc["static_poses"], np.float32).tobytes(), np.ascontiguousarray(sc["static_types"], np.int32).tobytes(),
                     np.ascontiguousarray(sc["static_geoms"], np.float32).tobytes(), np.stack([A, B], 1).astype(np.uint32).tobytes(),
                     pair_friction.tobytes(), params.tobytes()])
    out = subprocess.run([exe], input=blob, capture_output=True, check=True).stdout
    res = np.frombuffer(out[:n * 52], np.float32).reshape(n, 13)
    nc = int(np.frombuffer(out[n * 52:n * 52 + 4], np.uint32)[0])
    a, b, s, c, ct, mat = scene_contacts("orc", sc, A, B)
    assert nc == len(a) and nc > 0
    vel, pose, _, _, _ = run_tgs("orc", sc, a, b, s, c, ct, mat)
    assert velocity_error(vel, res[:, :6]) <= 1e-5
    assert np.abs(pose - res[:, 6:]).max() <= 1e-6
