"""libgbpx_immediate.so as a drop-in for the reference's immediate-mode TGS path.
Programs written against the reference's interface (PxGenerateContacts,
PxConstructSolverBodiesTGS, PxConstructStaticSolverBodyTGS,
PxBatchConstraintsTGS, PxCreateContactConstraintsTGS, PxSolveConstraintsTGS,
PxIntegrateSolverBodiesTGS) are linked against this library:

* tests/immediate_dropin.cpp, one frame with fresh caches, matches the CPU
  oracle's frame on the same scene;
* tests/immediate_contacts.cpp, PxGenerateContacts with PxCache memory kept
  between frames, matches the reference's own outputs (pcm_cached.npz), and
  with PxConvexCoreGeometry shapes (np_convex_core.npz);
* tests/immediate_dropin_frames.cpp, frames of one scene in the snippet's
  persistent mode (pair caches and friction data carried from frame to frame),
  matches the oracle's persistent frames step by step."""
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


def _build(tmp, name="immediate_dropin"):
    exe = os.path.join(tmp, name)
    lib_dir = os.path.join(ROOT, "physx_gb300")
    subprocess.check_call([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", name + ".cpp"), "-o", exe, "-L", lib_dir, "-lgbpx_immediate",
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


def test_immediate_cached_contacts_match_reference_golden(cuda_device, tmp_path):
    """PxGenerateContacts with caches kept between 8 moving frames: the reference's
    counts every frame and every value within the contact tolerance."""
    from contact_compare import CONTACT_TOL, unpack
    from test_oracle_golden import GOLDEN, load_np_cached_fixture
    exe = _build(str(tmp_path), "immediate_contacts")
    pairs, frames = load_np_cached_fixture(os.path.join(GOLDEN, "pcm_cached.npz"))
    n = len(pairs["type0"])
    geom = np.concatenate([np.asarray(pairs["geom0"], np.float32), np.asarray(pairs["geom1"], np.float32)], 1)
    blob = [np.array([n, len(frames)], np.uint32).tobytes(), np.asarray(pairs["type0"], np.int32).tobytes(),
            np.asarray(pairs["type1"], np.int32).tobytes(), np.ascontiguousarray(geom).tobytes()]
    for fr in frames:
        blob += [np.ascontiguousarray(fr["pose0"], np.float32).tobytes(), np.ascontiguousarray(fr["pose1"], np.float32).tobytes()]
    out = subprocess.run([exe], input=b"".join(blob), capture_output=True, check=True).stdout
    words = np.frombuffer(out, np.uint32)
    k = 0
    for f, fr in enumerate(frames):
        ref = unpack(fr["counts"], fr["contacts"])
        for i in range(n):
            c = int(words[k])
            k += 1
            assert c == fr["counts"][i], (f, i)
            got = words[k:k + 8 * c].view(np.float32).reshape(c, 8)
            k += 8 * c
            if c:
                assert np.abs(got[:, :7] - ref[i][:, :7]).max() <= CONTACT_TOL, (f, i)
    assert k == len(words)


def test_immediate_convex_core_contacts_match_reference_golden(cuda_device, tmp_path):
    """PxGenerateContacts of libgbpx_immediate.so with PxConvexCoreGeometry shapes
    (every core type against every shape type, np_convex_core.npz: the
    reference's own outputs): same counts, every value within the contact
    tolerance, and no cache memory kept for these pairs."""
    from contact_compare import CONTACT_TOL, unpack
    from test_oracle_golden import GOLDEN, load_np_fixture
    exe = _build(str(tmp_path), "immediate_contacts")
    pairs, rc, rpacked, _, _ = load_np_fixture(os.path.join(GOLDEN, "np_convex_core.npz"))
    n = len(pairs["type0"])
    geom = np.concatenate([np.asarray(pairs["geom0"], np.float32), np.asarray(pairs["geom1"], np.float32)], 1)
    blob = [np.array([n, 1], np.uint32).tobytes(), np.asarray(pairs["type0"], np.int32).tobytes(),
            np.asarray(pairs["type1"], np.int32).tobytes(), np.ascontiguousarray(geom).tobytes(),
            np.ascontiguousarray(pairs["pose0"], np.float32).tobytes(), np.ascontiguousarray(pairs["pose1"], np.float32).tobytes()]
    out = subprocess.run([exe], input=b"".join(blob), capture_output=True, check=True).stdout
    words = np.frombuffer(out, np.uint32)
    ref = unpack(rc, rpacked)
    k = 0
    for i in range(n):
        c = int(words[k])
        k += 1
        assert c == rc[i], i
        got = words[k:k + 8 * c].view(np.float32).reshape(c, 8)
        k += 8 * c
        if c:
            assert np.abs(got[:, :7] - ref[i][:, :7]).max() <= CONTACT_TOL, i
    assert k == len(words)


@pytest.mark.parametrize("batch", [True, False], ids=["batched", "one header per constraint"])
def test_immediate_pgs_frames_match_reference_golden(cuda_device, tmp_path, batch):
    """A program written against the reference's PGS interface (PxConstructSolverBodies,
    PxConstructStaticSolverBody, PxBatchConstraints, PxCreateContactConstraints,
    PxSolveConstraints, PxIntegrateSolverBodies; tests/immediate_pgs.cpp) linked
    against libgbpx_immediate.so reproduces the reference's PGS frames
    (pgs_*.npz): headers, types and order exactly, velocities, poses and the
    written-back normal impulses within the PGS bar of tests/test_pgs_gpu.py."""
    import glob
    import struct
    from test_oracle_golden import GOLDEN, load_tgs_fixture
    from test_pgs_gpu import assert_pgs_close
    exe = _build(str(tmp_path), "immediate_pgs")
    for path in sorted(glob.glob(os.path.join(GOLDEN, "pgs_*.npz"))):
        rb, z = load_tgs_fixture(path)
        n, m, nc, ncts = len(rb), len(z["static_poses"]), len(z["body_a"]), len(z["contacts"])
        blob = struct.pack("<5I", n, m, nc, ncts, 1 if batch else 0) + rb.tobytes() + np.ascontiguousarray(z["static_poses"], np.float32).tobytes()
        for k in ("body_a", "body_b", "contact_start", "contact_count"):
            blob += np.ascontiguousarray(z[k], np.uint32).tobytes()
        blob += np.ascontiguousarray(z["contacts"], np.float32).tobytes() + np.ascontiguousarray(z["material"], np.float32).tobytes()
        blob += struct.pack("<4f2I", 1.0 / 60.0, 0.0, -9.81, 0.0, 4, 1)
        out = subprocess.run([exe], input=blob, capture_output=True, check=True).stdout
        body = np.frombuffer(out[: n * 52], np.float32).reshape(n, 13)
        nh = struct.unpack_from("<I", out, n * 52)[0]
        off = n * 52 + 4
        hdr = np.frombuffer(out[off: off + nh * 12], np.uint32).reshape(nh, 3)
        off += nh * 12
        order = np.frombuffer(out[off: off + nc * 4], np.uint32)
        forces = np.frombuffer(out[off + nc * 4:], np.float32)
        got = dict(vel=body[:, :6].copy(), pose=body[:, 6:].copy(), header_start=hdr[:, 0].copy(), header_stride=hdr[:, 1].copy(),
                   header_type=hdr[:, 2].copy(), order=order.copy(), forces=forces.copy())
        tag = "batched" if batch else "single"
        ref = {k: z["ref_%s_%s" % (tag, k)] for k in ("vel", "pose", "header_start", "header_stride", "header_type", "order", "forces")}
        assert_pgs_close(ref, got, path)


def test_immediate_pgs_null_allocator_fails_cleanly(cuda_device, tmp_path):
    """A PxConstraintAllocator that returns null: PxCreateContactConstraints returns
    false (the program reports it and exits 3) instead of writing through it."""
    import glob
    import struct
    from test_oracle_golden import GOLDEN, load_tgs_fixture
    exe = _build(str(tmp_path), "immediate_pgs")
    path = sorted(glob.glob(os.path.join(GOLDEN, "pgs_*.npz")))[0]
    rb, z = load_tgs_fixture(path)
    n, m, nc, ncts = len(rb), len(z["static_poses"]), len(z["body_a"]), len(z["contacts"])
    blob = struct.pack("<5I", n, m, nc, ncts, 1) + rb.tobytes() + np.ascontiguousarray(z["static_poses"], np.float32).tobytes()
    for k in ("body_a", "body_b", "contact_start", "contact_count"):
        blob += np.ascontiguousarray(z[k], np.uint32).tobytes()
    blob += np.ascontiguousarray(z["contacts"], np.float32).tobytes() + np.ascontiguousarray(z["material"], np.float32).tobytes()
    blob += struct.pack("<4f2I", 1.0 / 60.0, 0.0, -9.81, 0.0, 4, 1)
    r = subprocess.run([exe, "nullalloc"], input=blob, capture_output=True)
    assert r.returncode == 3 and b"contact prep failed" in r.stderr


@pytest.mark.parametrize("seed", [121, 122])
def test_immediate_persistent_frames_match_oracle(cuda_device, tmp_path, seed):
    """Ten frames of a pile through the drop-in the way the snippet runs its
    persistent mode (PxCache per pair, friction data handed back through
    PxTGSSolverContactDesc::frictionPtr/frictionCount) against the oracle's
    persistent frames, frame by frame.  Each oracle frame starts from the bodies
    the drop-in wrote the frame before, while both sides keep their own pair state
    (caches, friction patches): the per-frame bar holds for the carried state, and
    the last-ulp differences of sin/cos in the integration (device libm against
    the host's) cannot grow over frames into a chaotic separation of the pile."""
    from oracle_libs import PersistentScenes
    from physx_gb300.world import DEFAULT_PARAMS
    from scenarios import pile_scenes
    from test_oracle_golden import rigid_velocity
    exe = _build(str(tmp_path), "immediate_dropin_frames")
    frames = 10
    sc = pile_scenes(seed, 1, 60)
    n, m = int(sc["body_count"][0]), int(sc["static_count"][0])
    p = DEFAULT_PARAMS
    params = np.array([p["dt"], *p["gravity"], p["contact_distance"], p["tolerance_length"], p["bounds_margin"], p["bounce_threshold"],
                       p["friction_offset_threshold"], p["correlation_distance"], p["static_friction"]], np.float32)
    blob = b"".join([np.array([n, m, frames], np.uint32).tobytes(), np.ascontiguousarray(sc["rigid"]).tobytes(),
                     np.ascontiguousarray(sc["types"], np.int32).tobytes(), np.ascontiguousarray(sc["geoms"], np.float32).tobytes(),
                     np.ascontiguousarray(sc["friction"], np.float32).tobytes(), np.ascontiguousarray(sc["static_poses"], np.float32).tobytes(),
                     np.ascontiguousarray(sc["static_types"], np.int32).tobytes(), np.ascontiguousarray(sc["static_geoms"], np.float32).tobytes(),
                     params.tobytes()])
    out = subprocess.run([exe], input=blob, capture_output=True, check=True).stdout
    rb_bytes = sc["rigid"].dtype.itemsize * n
    assert len(out) == frames * (rb_bytes + 4)
    orc = PersistentScenes("orc", sc, DEFAULT_PARAMS)
    for f in range(frames):
        chunk = out[f * (rb_bytes + 4):(f + 1) * (rb_bytes + 4)]
        got = np.frombuffer(chunk[:rb_bytes], sc["rigid"].dtype)
        assert int(np.frombuffer(chunk[rb_bytes:], np.uint32)[0]) > 0
        ref = orc.step().copy()
        orc.rb[:] = got
        assert velocity_error(rigid_velocity(ref), rigid_velocity(got)) <= 1e-5, f
        assert np.abs(got["p"] - ref["p"]).max() <= 1e-6, f
    orc.release()


def _bp_blob(mode, frames):
    parts = [np.array([mode, len(frames)], np.uint32).tobytes()]
    for fr in frames:
        cap = int(fr["capacity"])
        c, u, r = (np.ascontiguousarray(fr[k], np.uint32) for k in ("created", "updated", "removed"))
        parts += [np.array([cap, len(c), len(u), len(r)], np.uint32).tobytes(), c.tobytes(), u.tobytes(), r.tobytes()]
        bounds = np.zeros((cap + 1, 6), np.float32)
        b = np.asarray(fr["bounds"], np.float32)
        bounds[:min(len(b), cap + 1)] = b[:cap + 1]
        parts += [bounds.tobytes(), np.ascontiguousarray(fr["groups"][:cap], np.uint32).tobytes(),
                  np.ascontiguousarray(fr["distances"][:cap], np.float32).tobytes()]
    return b"".join(parts)


def _bp_results(out, nframes):
    res, off = [], 0
    for _ in range(nframes):
        nc, nl = np.frombuffer(out[off:off + 8], np.uint32)
        off += 8
        created = np.frombuffer(out[off:off + 8 * nc], np.uint32).reshape(-1, 2)
        off += 8 * nc
        lost = np.frombuffer(out[off:off + 8 * nl], np.uint32).reshape(-1, 2)
        off += 8 * nl
        res.append((created, lost))
    assert off == len(out)
    return res


@pytest.mark.parametrize("mode", [0, 1], ids=["PxBroadPhase", "PxAABBManager"])
@pytest.mark.parametrize("fixture", ["bp_dense.npz", "bp_sparse.npz"])
def test_immediate_broadphase_matches_reference_golden(cuda_device, tmp_path, fixture, mode):
    """tests/immediate_broadphase.cpp, written against PxBroadPhase.h, drives
    PxCreateBroadPhase(eABP) update / fetchResults with its own arrays from the
    broadphase's allocator (mode 0), or a PxAABBManager fed object by object
    (mode 1): the created and lost pairs of every frame equal the reference
    ABP's own (golden fixture), bit for bit."""
    from scenarios import sorted_pairs
    from test_oracle_golden import GOLDEN, load_bp_fixture
    exe = _build(str(tmp_path), "immediate_broadphase")
    frames = load_bp_fixture(os.path.join(GOLDEN, fixture))
    out = subprocess.run([exe], input=_bp_blob(mode, frames), capture_output=True, check=True).stdout
    for f, ((created, lost), fr) in enumerate(zip(_bp_results(out, len(frames)), frames)):
        assert np.array_equal(created, sorted_pairs(fr["ref_created"])), "frame %d created" % f
        assert np.array_equal(lost, sorted_pairs(fr["ref_lost"])), "frame %d lost" % f
