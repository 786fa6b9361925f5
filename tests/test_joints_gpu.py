"""GB300 joints (1D constraints): PxCreateJointConstraintsTGS and the joint half
of PxSolveConstraintsTGS against the reference's own joint frames
(tests/golden/joints_*.npz) and against the CPU oracle on seeded scenes:
headers, their per-pair / 4-wide types and the joint order exactly; body
velocities within 1e-5 relative (per body, against max(|v|, 1e-2)), poses
within 2e-6, write-back impulses within 1e-5 relative (per joint, against
max(|impulse|, 1e-2)) and broken flags exactly.  (The body integration
evaluates sine and cosine with the device's functions, so poses and the
velocities that follow them differ from the CPU by rounding only.)"""
import glob
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from joint_scenes import joint_frame, load_joint_fixture, make_joint_scene
from oracle_libs import advance_rigid, run_joints
from test_oracle_golden import velocity_error

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
JOINT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "joints_*.npz")))


def impulse_error(ref, got):
    lin = np.linalg.norm(ref[:, :3], axis=1)
    ang = np.linalg.norm(ref[:, 3:], axis=1)
    scale = np.maximum(np.stack([lin] * 3 + [ang] * 3, 1), 1e-2)
    return float((np.abs(ref - got) / scale).max()) if len(ref) else 0.0


def assert_frame_close(ref, got, what):
    for k in ("header_start", "header_stride", "header_type", "order", "broken"):
        assert np.array_equal(got[k], ref[k]), "%s: %s" % (what, k)
    assert velocity_error(ref["vel"], got["vel"]) <= 1e-5, what
    assert np.abs(ref["pose"] - got["pose"]).max() <= 2e-6, what
    assert impulse_error(ref["force"], got["force"]) <= 1e-5, what


@pytest.mark.parametrize("path", JOINT_FIXTURES, ids=[os.path.basename(p) for p in JOINT_FIXTURES])
def test_joint_frames_match_reference_golden(cuda_device, path):
    from physx_gb300.solver import joint_frame as gpu_joint_frame
    for fr in load_joint_fixture(path):
        ref = {k: fr["ref_" + k] for k in ("vel", "pose", "header_start", "header_stride", "header_type", "order", "force", "broken")}
        assert_frame_close(ref, gpu_joint_frame(fr), "frame %d" % fr["frame"])


@pytest.mark.parametrize("seed,batch", [(41, True), (42, False), (43, True)])
def test_joint_frames_match_oracle(cuda_device, seed, batch):
    """25 consecutive frames of a seeded joint scene, each frame's rows written
    from the poses the oracle's previous frame left: the GB300 frame against the
    oracle's on the same inputs."""
    from physx_gb300.solver import joint_frame as gpu_joint_frame
    sc = make_joint_scene(seed, nb_chains=10, links=(2, 8))
    rigid = sc["rigid"]
    for f in range(25):
        fr = joint_frame(sc, rigid)
        ref = run_joints("orc", fr, batch=batch)
        assert_frame_close(ref, gpu_joint_frame(fr, batch=batch), "frame %d" % f)
        rigid = advance_rigid(rigid, ref["vel"], ref["pose"])


def _build(tmp):
    exe = os.path.join(tmp, "immediate_joints")
    lib_dir = os.path.join(ROOT, "physx_gb300")
    subprocess.check_call([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "immediate_joints.cpp"), "-o", exe, "-L", lib_dir, "-lgbpx_immediate",
                           "-Wl,-rpath," + lib_dir])
    return exe


def _run_dropin(exe, fr, batch, dt=1.0 / 60.0, gravity=(0.0, -9.81, 0.0), nb_pos=4, nb_vel=1, shader=False):
    n, nj = int(fr["nb_dyn"]), len(fr["joint_a"])
    rows = np.ascontiguousarray(fr["rows"])
    blob = struct.pack("<5I", n, len(fr["static_poses"]), nj, len(rows), 1 if batch else 0)
    blob += np.ascontiguousarray(fr["rigid"]).tobytes() + np.ascontiguousarray(fr["static_poses"], np.float32).tobytes()
    for k in ("joint_a", "joint_b", "row_start", "row_count"):
        blob += np.ascontiguousarray(fr[k], np.uint32).tobytes()
    blob += rows.tobytes() + np.ascontiguousarray(fr["params"], np.float32).tobytes()
    blob += struct.pack("<4f2I", dt, *gravity, nb_pos, nb_vel)
    out = subprocess.run([exe] + (["shader"] if shader else []), input=blob, capture_output=True, check=True).stdout
    body = np.frombuffer(out[: n * 52], np.float32).reshape(n, 13)
    nh = struct.unpack_from("<I", out, n * 52)[0]
    hdr = np.frombuffer(out[n * 52 + 4: n * 52 + 4 + nh * 12], np.uint32).reshape(nh, 3)
    rest = out[n * 52 + 4 + nh * 12:]
    per = np.frombuffer(rest, np.uint8).reshape(nj, 28)
    force = per[:, :24].copy().view(np.float32).reshape(nj, 6)
    broken = per[:, 24:].copy().view(np.uint32).reshape(nj)
    return dict(vel=body[:, :6].copy(), pose=body[:, 6:].copy(), header_start=hdr[:, 0].copy(), header_stride=hdr[:, 1].copy(),
                header_type=hdr[:, 2].copy(), force=force, broken=broken)


@pytest.mark.parametrize("batch", [True, False], ids=["batched", "per-joint headers"])
def test_immediate_joints_match_reference_golden(cuda_device, tmp_path, batch):
    """A program written against the reference's interface (PxBatchConstraintsTGS,
    PxCreateJointConstraintsTGS, PxSolveConstraintsTGS with the write-back of
    PxTGSSolverConstraintPrepDesc::writeback) linked against
    libgbpx_immediate.so: batched, it reproduces the reference's frames of the
    joints_chains fixture; with one header per joint, the oracle's."""
    exe = _build(str(tmp_path))
    for fr in load_joint_fixture(os.path.join(GOLDEN, "joints_chains.npz")):
        if batch:
            ref = {k: fr["ref_" + k] for k in ("vel", "pose", "header_start", "header_stride", "header_type", "force", "broken")}
        else:
            ref = run_joints("orc", fr, batch=False)
        got = _run_dropin(exe, fr, batch)
        for k in ("header_start", "header_stride", "header_type", "broken"):
            assert np.array_equal(got[k], ref[k]), "frame %d %s" % (fr["frame"], k)
        assert velocity_error(ref["vel"], got["vel"]) <= 1e-5
        assert np.abs(ref["pose"] - got["pose"]).max() <= 2e-6
        assert impulse_error(ref["force"], got["force"]) <= 1e-5


def test_immediate_joint_shaders_match_reference_golden(cuda_device, tmp_path):
    """The same program with its rows returned by an immediate joint shader
    (PxImmediateConstraint; PxCreateJointConstraintsWithImmediateShadersTGS,
    PxImmediateMode.h:696): the shader also sets the mass scales, the constraint
    frames and body 0's offset, and the frames equal the reference's."""
    exe = _build(str(tmp_path))
    for fr in load_joint_fixture(os.path.join(GOLDEN, "joints_chains.npz")):
        ref = {k: fr["ref_" + k] for k in ("vel", "pose", "header_start", "header_stride", "header_type", "force", "broken")}
        got = _run_dropin(exe, fr, True, shader=True)
        for k in ("header_start", "header_stride", "header_type", "broken"):
            assert np.array_equal(got[k], ref[k]), "frame %d %s" % (fr["frame"], k)
        assert velocity_error(ref["vel"], got["vel"]) <= 1e-5
        assert np.abs(ref["pose"] - got["pose"]).max() <= 2e-6
        assert impulse_error(ref["force"], got["force"]) <= 1e-5
