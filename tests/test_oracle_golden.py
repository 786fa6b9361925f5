"""The CPU oracle (oracle/port) against the reference's own outputs.

Golden fixtures in tests/golden were produced by the reference built from its
sources (tests/golden/make_golden.py).  Where that build is present (the
development machine), extra seeded cases are also compared live."""
import glob
import os

import numpy as np
import pytest

from oracle_libs import CpuBroadPhase, reference
from scenarios import bp_frames, sorted_pairs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_bp_fixture(path):
    z = np.load(path)
    frames = []
    for f in range(int(z["frames"])):
        fr = {k: z["f%d_%s" % (f, k)] for k in ("created", "updated", "removed", "bounds", "groups", "distances")}
        fr["capacity"] = int(z["f%d_capacity" % f])
        fr["ref_created"] = z["f%d_ref_created" % f]
        fr["ref_lost"] = z["f%d_ref_lost" % f]
        frames.append(fr)
    return frames


BP_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "bp_*.npz")))


@pytest.mark.parametrize("path", BP_FIXTURES, ids=[os.path.basename(p) for p in BP_FIXTURES])
def test_oracle_bp_matches_reference_golden(path):
    bp = CpuBroadPhase("orc")
    for f, fr in enumerate(load_bp_fixture(path)):
        created, lost = bp.update(fr)
        assert np.array_equal(sorted_pairs(created), sorted_pairs(fr["ref_created"])), "frame %d created" % f
        assert np.array_equal(sorted_pairs(lost), sorted_pairs(fr["ref_lost"])), "frame %d lost" % f
    bp.release()


def test_bp_fixtures_present():
    assert len(BP_FIXTURES) >= 2


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,n,frames,extent", [(21, 3000, 5, 40.0), (22, 200, 10, 5.0)])
def test_oracle_bp_matches_reference_live(seed, n, frames, extent):
    ref, orc = CpuBroadPhase("pxref"), CpuBroadPhase("orc")
    for fr in bp_frames(seed, n, frames, extent=extent):
        rc, rl = ref.update(fr)
        oc, ol = orc.update(fr)
        assert np.array_equal(sorted_pairs(rc), sorted_pairs(oc))
        assert np.array_equal(sorted_pairs(rl), sorted_pairs(ol))


NP_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "np_*.npz")))


def load_np_fixture(path):
    z = np.load(path)
    pairs = {k: z[k] for k in ("type0", "geom0", "type1", "geom1", "pose0", "pose1")}
    return pairs, z["counts"], z["contacts"], float(z["contact_distance"]), float(z["tolerance_length"])


@pytest.mark.parametrize("path", NP_FIXTURES, ids=[os.path.basename(p) for p in NP_FIXTURES])
def test_oracle_contacts_match_reference_golden(path):
    from contact_compare import assert_report, compare, unpack
    from oracle_libs import run_contacts
    pairs, rc, rpacked, cd, tl = load_np_fixture(path)
    oc, oo = run_contacts("orc", pairs, contact_distance=cd, tolerance_length=tl, max_per_pair=8)
    rep = compare(pairs, rc, unpack(rc, rpacked), oc, [oo[i, :oc[i]] for i in range(len(oc))])
    assert_report(rep)
    # every pair kind, including the GJK/EPA paths, is reproduced bit for bit
    if "convex" in os.path.basename(path):
        kinds = [k for k in rep if "convex_" in k]
        for core in ("point", "segment", "box", "ellipsoid", "cylinder", "cone"):
            for other in ("sphere", "plane", "capsule", "box", "convex_point"):
                assert any(k in ("%s-convex_%s" % (other, core), "convex_%s-%s" % (core, other)) for k in kinds), (core, other)
    else:
        kinds = ("sphere-sphere", "sphere-plane", "sphere-capsule", "sphere-box", "plane-capsule", "plane-box", "capsule-capsule",
                 "capsule-box", "box-box")
    for k in kinds:
        assert rep[k]["maxdiff"] == 0.0, (k, rep[k])


def test_oracle_recip_fast_matches_reference_golden():
    """The approximate reciprocal of the box-box edge clipping (V3RecipFast) against
    the reference's own outputs: one input per 2^-11 mantissa cell plus random and
    special values."""
    import ctypes
    from oracle_libs import oracle
    z = np.load(os.path.join(GOLDEN, "recip_fast.npz"))
    x = np.ascontiguousarray(z["x"], np.float32)
    out = np.zeros_like(x)
    oracle().orc_recip_fast(x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(len(x)))
    assert np.array_equal(out.view(np.uint32), z["ref"].view(np.uint32))


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,types", [(51, None), (52, [(2, 3), (3, 2), (3, 3)])])
def test_oracle_contacts_match_reference_live(seed, types):
    from contact_compare import assert_report, compare
    from oracle_libs import run_contacts
    from scenarios import np_pairs
    pairs = np_pairs(seed, 6000, types=types)
    rc, ro = run_contacts("pxref", pairs, max_per_pair=8)
    oc, oo = run_contacts("orc", pairs, max_per_pair=8)
    rep = compare(pairs, rc, [ro[i, :rc[i]] for i in range(len(rc))], oc, [oo[i, :oc[i]] for i in range(len(oc))])
    assert_report(rep)
    assert all(r["maxdiff"] == 0.0 for r in rep.values()), rep


def load_np_cached_fixture(path):
    """The pairs, and per frame their poses with the reference's counts and packed contacts."""
    z = np.load(path)
    pairs = {k: z[k] for k in ("type0", "geom0", "type1", "geom1")}
    frames = [dict(pose0=z["f%d_pose0" % f], pose1=z["f%d_pose1" % f], counts=z["f%d_counts" % f], contacts=z["f%d_contacts" % f])
              for f in range(int(z["frames"]))]
    return pairs, frames


def test_oracle_cached_contacts_match_reference_golden():
    """PxGenerateContacts with persistent caches (the PCM manifold of plane-capsule,
    plane-box, capsule-box and box-box pairs carried between frames: refresh,
    invalidation, incremental points, GJK warm start) over 8 moving frames."""
    from contact_compare import unpack
    from oracle_libs import CachedContacts
    pairs, frames = load_np_cached_fixture(os.path.join(GOLDEN, "pcm_cached.npz"))
    n = len(pairs["type0"])
    orc = CachedContacts("orc", n)
    for f, fr in enumerate(frames):
        oc, oo = orc.run(dict(pairs, pose0=fr["pose0"], pose1=fr["pose1"]))
        assert np.array_equal(oc, fr["counts"]), "frame %d counts" % f
        ref = unpack(fr["counts"], fr["contacts"])
        for i in range(n):
            assert np.array_equal(oo[i, :oc[i]], ref[i]), "frame %d pair %d" % (f, i)


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed", [63, 64])
def test_oracle_cached_contacts_match_reference_live(seed):
    from oracle_libs import CachedContacts
    from scenarios import moving_pairs
    pairs, poses = moving_pairs(seed, 1400, 10)
    orc, ref = CachedContacts("orc", 1400), CachedContacts("pxref", 1400)
    for p0, p1 in poses:
        fr = dict(pairs, pose0=p0, pose1=p1)
        oc, oo = orc.run(fr)
        rc, ro = ref.run(fr)
        assert np.array_equal(oc, rc) and np.array_equal(oo, ro)
    ref.release()


TGS_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "tgs_*.npz")))

# Velocity tolerance of one TGS solve against the reference, relative to the
# body's speed (floor 1e-2 m/s), and pose tolerance (absolute).  The oracle
# restates both of the reference's contact paths (per-pair rows, and the 4-wide
# block path of DyTGSContactPrepBlock.cpp:1398 / solveContact4_Block :2280 for
# headers of stride 4) in the reference's evaluation order, so the oracle is
# held to exact equality; the device code is held to these bounds.
TGS_VEL_REL_TOL = 1e-5
TGS_POSE_TOL = 1e-6


def load_tgs_fixture(path):
    z = np.load(path)
    from scenarios import rigid_body_data
    rb = rigid_body_data(len(z["rigid"]))
    rb.view(np.uint8).reshape(len(rb), 96)[:] = z["rigid"]
    return rb, {k: z[k] for k in z.files if k != "rigid"}


def velocity_error(ref, got):
    lin = np.linalg.norm(ref[:, :3], axis=1)
    ang = np.linalg.norm(ref[:, 3:], axis=1)
    scale = np.maximum(np.stack([lin] * 3 + [ang] * 3, 1), 1e-2)
    return float((np.abs(ref - got) / scale).max())


@pytest.mark.parametrize("path", TGS_FIXTURES, ids=[os.path.basename(p) for p in TGS_FIXTURES])
def test_oracle_tgs_matches_reference_golden(path):
    from oracle_libs import run_tgs
    rb, z = load_tgs_fixture(path)
    sc = dict(types=np.zeros(len(rb), np.int32), rigid=rb, static_poses=z["static_poses"])
    vel, pose, hs, hst, order = run_tgs("orc", sc, z["body_a"], z["body_b"], z["contact_start"], z["contact_count"], z["contacts"],
                                        z["material"])
    # batching is reproduced exactly
    assert np.array_equal(hs, z["ref_header_start"]) and np.array_equal(hst, z["ref_header_stride"])
    assert np.array_equal(order, z["ref_order"])
    assert np.array_equal(vel, z["ref_velocity"]) and np.array_equal(pose, z["ref_pose"])


PGS_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "pgs_*.npz")))
PGS_KEYS = ("vel", "pose", "header_start", "header_stride", "header_type", "order", "forces")


def pgs_fixture_args(path):
    rb, z = load_tgs_fixture(path)
    sc = dict(types=np.zeros(len(rb), np.int32), rigid=rb, static_poses=z["static_poses"])
    return sc, z, (z["body_a"], z["body_b"], z["contact_start"], z["contact_count"], z["contacts"], z["material"])


@pytest.mark.parametrize("batch", [True, False], ids=["batched", "one header per constraint"])
@pytest.mark.parametrize("path", PGS_FIXTURES, ids=[os.path.basename(p) for p in PGS_FIXTURES])
def test_oracle_pgs_matches_reference_golden(path, batch):
    """One PGS frame (PxConstructSolverBodies, PxBatchConstraints,
    PxCreateContactConstraints, PxSolveConstraints, PxIntegrateSolverBodies):
    velocities, poses, headers with their types, the order and the
    written-back normal impulses equal the reference's bit for bit, with the
    4-wide block path (batched) and the per-pair path."""
    from oracle_libs import run_pgs
    sc, z, args = pgs_fixture_args(path)
    got = run_pgs("orc", sc, *args, batch=batch)
    tag = "batched" if batch else "single"
    for k in PGS_KEYS:
        assert np.array_equal(got[k], z["ref_%s_%s" % (tag, k)]), k
    if batch:
        assert {6, 7} & set(got["header_type"].tolist())   # block headers are in the fixture


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,n,restitution,iters", [(61, 40, 0.0, (4, 1)), (62, 200, 0.3, (4, 1)), (63, 120, 0.0, (8, 2)), (64, 60, 0.5, (1, 1))])
def test_oracle_pgs_matches_reference_live(seed, n, restitution, iters):
    from oracle_libs import run_pgs, scene_contacts, scene_pairs
    from scenarios import random_scene
    sc = random_scene(seed, n)
    A, B = scene_pairs(sc)
    a, b, s, c, ct, mat = scene_contacts("pxref", sc, A, B)
    mat[:, 2] = restitution
    for batch in (True, False):
        r = run_pgs("pxref", sc, a, b, s, c, ct, mat, batch=batch, nb_pos=iters[0], nb_vel=iters[1])
        o = run_pgs("orc", sc, a, b, s, c, ct, mat, batch=batch, nb_pos=iters[0], nb_vel=iters[1])
        for k in PGS_KEYS:
            assert np.array_equal(r[k], o[k]), (batch, k)


SCENE_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "scene_*.npz")))


def load_scene_fixture(path):
    from scenarios import rigid_body_data
    z = np.load(path)
    rb = rigid_body_data(len(z["rigid"]))
    rb.view(np.uint8).reshape(len(rb), 96)[:] = z["rigid"]
    ref = rigid_body_data(len(z["rigid"]))
    ref.view(np.uint8).reshape(len(ref), 96)[:] = z["ref_rigid"]
    scenes = {k: z[k] for k in z.files if k not in ("rigid", "ref_rigid")}
    scenes["rigid"] = rb
    return scenes, ref


def rigid_velocity(rb):
    return np.concatenate([rb["linVel"], rb["angVel"]], axis=1)


@pytest.mark.parametrize("path", SCENE_FIXTURES, ids=[os.path.basename(p) for p in SCENE_FIXTURES])
def test_oracle_scene_step_matches_reference_golden(path):
    from oracle_libs import run_scene_step
    sys_path_root()
    from physx_gb300.world import DEFAULT_PARAMS
    scenes, ref = load_scene_fixture(path)
    out = run_scene_step("orc", scenes, DEFAULT_PARAMS, steps=1)
    assert np.array_equal(rigid_velocity(ref), rigid_velocity(out))
    assert np.array_equal(out["p"], ref["p"]) and np.array_equal(out["q"], ref["q"])


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed", [100, 101, 102])
def test_oracle_scene_steps_match_reference_live(seed):
    """Mixed sphere/capsule/box piles, 20 frames: the oracle equals the reference bit for bit."""
    from oracle_libs import run_scene_step
    from scenarios import pile_scenes
    sys_path_root()
    from physx_gb300.world import DEFAULT_PARAMS
    sc = pile_scenes(seed, 3, 60)
    a = run_scene_step("orc", sc, DEFAULT_PARAMS, steps=20)
    b = run_scene_step("pxref", sc, DEFAULT_PARAMS, steps=20)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def load_persistent_fixture(path):
    from scenarios import rigid_body_data
    z = np.load(path)
    rb = rigid_body_data(len(z["rigid"]))
    rb.view(np.uint8).reshape(len(rb), 96)[:] = z["rigid"]
    frames = []
    for f in range(int(z["frames"])):
        r = rigid_body_data(len(z["rigid"]))
        r.view(np.uint8).reshape(len(r), 96)[:] = z["ref_rigid_%d" % f]
        frames.append(r)
    scenes = {k: z[k] for k in z.files if k != "rigid" and k != "frames" and not k.startswith("ref_rigid_")}
    scenes["rigid"] = rb
    return scenes, frames


PERSISTENT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "persist_*.npz")))


@pytest.mark.parametrize("path", PERSISTENT_FIXTURES, ids=[os.path.basename(p) for p in PERSISTENT_FIXTURES])
def test_oracle_persistent_frames_match_reference_golden(path):
    """Frames with persistent pair state (PCM caches and friction patches carried
    between frames, broken-friction flags, block-path patch handling): every frame
    equals the reference's bit for bit."""
    from oracle_libs import PersistentScenes
    sys_path_root()
    from physx_gb300.world import DEFAULT_PARAMS
    scenes, frames = load_persistent_fixture(path)
    orc = PersistentScenes("orc", scenes, DEFAULT_PARAMS)
    for f, ref in enumerate(frames):
        out = orc.step()
        assert np.array_equal(out.view(np.uint8), ref.view(np.uint8)), "frame %d" % f
    orc.release()


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed", [210, 211])
def test_oracle_persistent_frames_match_reference_live(seed):
    from oracle_libs import PersistentScenes
    from scenarios import pile_scenes
    sys_path_root()
    from physx_gb300.world import DEFAULT_PARAMS
    sc = pile_scenes(seed, 3, 60)
    orc, ref = PersistentScenes("orc", sc, DEFAULT_PARAMS), PersistentScenes("pxref", sc, DEFAULT_PARAMS)
    for _ in range(30):
        assert np.array_equal(orc.step().view(np.uint8), ref.step().view(np.uint8))
    orc.release()
    ref.release()


def sys_path_root():
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)


def test_oracle_large_scene_trace_equals_reference():
    """The oracle's 600-step trace of the 100k-body single-scene workload
    (tests/golden/make_large_trace.py run with the oracle) is the reference's,
    statistic for statistic: the restatement is pinned on the large-scene frame
    as well as on the small fixtures."""
    ref = np.load(os.path.join(GOLDEN, "large_scene_trace.npz"))
    orc = np.load(os.path.join(GOLDEN, "large_scene_trace_orc.npz"))
    assert int(ref["checksum"]) == int(orc["checksum"])
    assert np.array_equal(ref["stats"], orc["stats"])


JOINT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "joints_*.npz")))
JOINT_KEYS = ("vel", "pose", "header_start", "header_stride", "header_type", "order", "force", "broken")


def test_joint_fixtures_present():
    assert len(JOINT_FIXTURES) >= 2


@pytest.mark.parametrize("path", JOINT_FIXTURES, ids=[os.path.basename(p) for p in JOINT_FIXTURES])
def test_oracle_joints_match_reference_golden(path):
    """PxCreateJointConstraintsTGS + PxSolveConstraintsTGS on the reference's
    joint frames: headers (with their per-pair / 4-wide types), order,
    velocities, poses, write-back impulses and broken flags, bit for bit."""
    from joint_scenes import load_joint_fixture
    from oracle_libs import run_joints
    for fr in load_joint_fixture(path):
        got = run_joints("orc", fr)
        for k in JOINT_KEYS:
            assert np.array_equal(got[k], fr["ref_" + k]), "frame %d %s" % (fr["frame"], k)


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,batch", [(31, True), (32, False), (33, True)])
def test_oracle_joints_match_reference_live(seed, batch):
    """30 consecutive frames of a seeded joint scene (each frame's rows written
    from the poses the previous one left), the oracle against the reference."""
    from joint_scenes import joint_frame, make_joint_scene
    from oracle_libs import advance_rigid, run_joints
    sc = make_joint_scene(seed, nb_chains=8, links=(2, 7))
    rigid = sc["rigid"]
    for f in range(30):
        fr = joint_frame(sc, rigid)
        ref = run_joints("pxref", fr, batch=batch)
        got = run_joints("orc", fr, batch=batch)
        for k in JOINT_KEYS:
            assert np.array_equal(got[k], ref[k]), "frame %d %s" % (f, k)
        rigid = advance_rigid(rigid, ref["vel"], ref["pose"])


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,n,frames,extent", [(51, 3000, 6, 40.0), (52, 400, 8, 6.0)])
def test_reference_pabp_pairs_equal_abp(seed, n, frames, extent):
    """PxCreateBroadPhase(ePABP) gives the same created / lost pair sets as eABP
    frame by frame (the reference's own two broadphases), so serving ePABP
    descriptors with the ABP-exact device broadphase keeps ePABP's results."""
    abp, pabp = CpuBroadPhase("pxref"), CpuBroadPhase("pxref", pabp=True)
    for f, fr in enumerate(bp_frames(seed, n, frames, extent=extent)):
        ac, al = abp.update(fr)
        pc, pl = pabp.update(fr)
        assert np.array_equal(sorted_pairs(ac), sorted_pairs(pc)), "frame %d created" % f
        assert np.array_equal(sorted_pairs(al), sorted_pairs(pl)), "frame %d lost" % f
