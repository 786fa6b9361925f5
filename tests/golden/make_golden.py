"""Generates the golden fixtures in tests/golden/ by running the REFERENCE
(PhysX built from its own sources by oracle/ref/Makefile into
oracle/_ref/libpxref.so) on seeded synthetic inputs.

Run on the development machine, where the reference sources exist:

    make -C oracle/ref -j8 && python tests/golden/make_golden.py

Each fixture stores its inputs and the reference's outputs, so the tests on
machines without the reference need neither the reference nor this script.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle_libs import CachedContacts, CpuBroadPhase, PersistentScenes, reference, run_contacts, run_pgs, run_scene_step, run_tgs, scene_contacts, scene_pairs  # noqa: E402
from scenarios import bp_frames, moving_pairs, np_pairs, pile_scenes, random_scene  # noqa: E402
from physx_gb300.workloads import convex_core_pairs  # noqa: E402

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
    # name, seed, pairs, generator
    # near-contact pairs of every sphere/plane/capsule/box combination
    ("np_mixed", 17, 3000, np_pairs),
    # pairs with a convex core (PxConvexCoreGeometry, every core type) against every shape type
    ("np_convex_core", 19, 3000, lambda seed, n: convex_core_pairs(seed, n, aligned_frac=0.6)),
]


def make_np():
    for name, seed, n, gen in NP_CASES:
        pairs = gen(seed, n)
        cnt, out = run_contacts("pxref", pairs, max_per_pair=8)
        packed = np.concatenate([out[i, :cnt[i]] for i in range(n) if cnt[i]]) if cnt.sum() else np.zeros((0, 8), np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), counts=cnt, contacts=packed.astype(np.float32),
                            contact_distance=np.float32(0.04), tolerance_length=np.float32(1.0), **pairs)
        print("wrote", name)


NP_CACHED_CASES = [
    # name, seed, pairs, frames: the cached pair kinds moving a little every frame
    ("pcm_cached", 18, 630, 8),
]


def make_np_cached():
    for name, seed, n, frames in NP_CACHED_CASES:
        pairs, poses = moving_pairs(seed, n, frames)
        ref = CachedContacts("pxref", n)
        out = dict(frames=np.array(frames), contact_distance=np.float32(0.04), tolerance_length=np.float32(1.0),
                   **{k: pairs[k] for k in ("type0", "geom0", "type1", "geom1")})
        for f, (p0, p1) in enumerate(poses):
            cnt, res = ref.run(dict(pairs, pose0=p0, pose1=p1))
            out["f%d_pose0" % f], out["f%d_pose1" % f] = p0, p1
            out["f%d_counts" % f] = cnt
            out["f%d_contacts" % f] = (np.concatenate([res[i, :cnt[i]] for i in range(n) if cnt[i]]) if cnt.sum()
                                        else np.zeros((0, 8), np.float32))
        ref.release()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)


TGS_CASES = [
    # name, seed, bodies: a settled-looking pile of spheres/capsules/boxes on a plane
    ("tgs_pile_small", 31, 24),
    ("tgs_pile", 32, 160),
]


def make_tgs():
    for name, seed, n in TGS_CASES:
        sc = random_scene(seed, n)
        A, B = scene_pairs(sc)
        a, b, s_, c, ct, mat = scene_contacts("pxref", sc, A, B)
        vel, pose, hs, hst, order = run_tgs("pxref", sc, a, b, s_, c, ct, mat)
        L = reference()
        bv = np.zeros((n, 16), np.float32)
        btx = np.zeros((n, 16), np.float32)
        bd = np.zeros((n, 12), np.float32)
        g = np.array([0.0, -9.81, 0.0], np.float32)
        P = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        L.pxref_construct_bodies_tgs(P(sc["rigid"]), ctypes.c_uint32(n), P(g), ctypes.c_float(1.0 / 60.0), P(bv), P(btx), P(bd))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rigid=sc["rigid"].view(np.uint8).reshape(n, 96),
                            static_poses=sc["static_poses"], body_a=a, body_b=b, contact_start=s_, contact_count=c,
                            contacts=ct, material=mat, ref_velocity=vel, ref_pose=pose, ref_header_start=hs,
                            ref_header_stride=hst, ref_order=order, ref_body_vel=bv, ref_body_txi=btx, ref_body_data=bd)
        print("wrote", name)


PGS_CASES = [
    # name, seed, bodies, restitution: one PGS frame (PxConstructSolverBodies, PxBatchConstraints,
    # PxCreateContactConstraints with the 4-wide block path and the per-pair path, PxSolveConstraints,
    # PxIntegrateSolverBodies) with the batching and with one header per constraint
    ("pgs_pile", 51, 160, 0.0),
    ("pgs_pile_bouncy", 52, 80, 0.4),
]


def make_pgs():
    out_keys = ("vel", "pose", "header_start", "header_stride", "header_type", "order", "forces")
    for name, seed, n, rest in PGS_CASES:
        sc = random_scene(seed, n)
        A, B = scene_pairs(sc)
        a, b, s_, c, ct, mat = scene_contacts("pxref", sc, A, B)
        mat[:, 2] = rest
        out = dict(rigid=sc["rigid"].view(np.uint8).reshape(n, 96), static_poses=sc["static_poses"], body_a=a, body_b=b,
                   contact_start=s_, contact_count=c, contacts=ct, material=mat)
        for tag, batch in (("batched", True), ("single", False)):
            r = run_pgs("pxref", sc, a, b, s_, c, ct, mat, batch=batch)
            for k in out_keys:
                out["ref_%s_%s" % (tag, k)] = r[k]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)


SCENE_CASES = [
    # name, seed, scenes, bodies per scene, shapes: one full frame (bounds, ABP, contacts, TGS) per scene
    ("scene_spheres_capsules", 41, 4, 48, (0, 2)),
    ("scene_mixed", 42, 4, 40, (0, 2, 3)),
    ("scene_boxes", 43, 4, 32, (3,)),
]


def make_scene():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from physx_gb300.world import DEFAULT_PARAMS
    for name, seed, S, n, shapes in SCENE_CASES:
        sc = pile_scenes(seed, S, n, shapes=shapes)
        out = run_scene_step("pxref", sc, DEFAULT_PARAMS, steps=1)
        arrays = {k: v for k, v in sc.items() if k != "rigid"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rigid=sc["rigid"].view(np.uint8).reshape(-1, 96),
                            ref_rigid=out.view(np.uint8).reshape(-1, 96), **arrays)
        print("wrote", name)


PERSISTENT_CASES = [
    # name, seed, scenes, bodies per scene, frames: contact caches and friction data carried between frames
    ("persist_piles", 44, 3, 48, 24),
]


def make_persistent():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from physx_gb300.world import DEFAULT_PARAMS
    for name, seed, S, n, frames in PERSISTENT_CASES:
        sc = pile_scenes(seed, S, n)
        ref = PersistentScenes("pxref", sc, DEFAULT_PARAMS)
        out = {}
        for f in range(frames):
            out["ref_rigid_%d" % f] = ref.step().view(np.uint8).reshape(-1, 96).copy()
        ref.release()
        arrays = {k: v for k, v in sc.items() if k != "rigid"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rigid=sc["rigid"].view(np.uint8).reshape(-1, 96), frames=np.array(frames),
                            **out, **arrays)
        print("wrote", name)


def make_recip():
    """The reference's approximate reciprocal (V3RecipFast): one input per 2^-11
    mantissa cell of [1, 2), random magnitudes of both signs, and special values."""
    rng = np.random.default_rng(61)
    cells = (np.arange(2048, dtype=np.uint32) << 12) | np.uint32(0x3F800000)
    rnd = rng.uniform(-40.0, 40.0, 20000)
    x = np.concatenate([cells.view(np.float32), (np.sign(rng.standard_normal(20000)) * np.exp2(rnd)).astype(np.float32),
                        np.array([0.0, -0.0, np.inf, -np.inf, 1e-40, -1e-40, 3e38, -3e38, 1e-6, 1.0], np.float32)])
    x = np.ascontiguousarray(x, np.float32)
    ref = np.zeros_like(x)
    reference().pxref_recip_fast(x.ctypes.data_as(ctypes.c_void_p), ref.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(len(x)))
    np.savez_compressed(os.path.join(HERE, "recip_fast.npz"), x=x, ref=ref)
    print("wrote recip_fast")


def pyramid_trace(which, steps=300, persistent=False):
    """Long-horizon statistics of the 210-box pyramid stepped `steps` times: kinetic
    energy and highest / lowest box centre per step, final horizontal drift."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from physx_gb300.workloads import kinetic_energy, pyramid_scene
    from physx_gb300.world import DEFAULT_PARAMS
    sc = pyramid_scene()
    rb = sc["rigid"].copy()
    ke, top, low = [], [], []
    ps = PersistentScenes(which, sc, DEFAULT_PARAMS) if persistent else None
    for _ in range(steps):
        rb = ps.step().copy() if ps else run_scene_step(which, dict(sc, rigid=rb), DEFAULT_PARAMS, steps=1)
        ke.append(kinetic_energy(rb))
        top.append(float(rb["p"][:, 1].max()))
        low.append(float(rb["p"][:, 1].min()))
    drift = float(np.abs(rb["p"][:, 0] - sc["rigid"]["p"][:, 0]).mean())
    return dict(ke=np.array(ke), top=np.array(top), low=np.array(low), drift=np.float64(drift))


def make_pyramid():
    np.savez_compressed(os.path.join(HERE, "pyramid_stats.npz"), **pyramid_trace("pxref"))
    print("wrote pyramid_stats")
    np.savez_compressed(os.path.join(HERE, "pyramid_stats_persistent.npz"), **pyramid_trace("pxref", persistent=True))
    print("wrote pyramid_stats_persistent")


if __name__ == "__main__":
    if reference() is None:
        sys.exit("oracle/_ref/libpxref.so is missing: build it with make -C oracle/ref")
    which = sys.argv[1:] or ["bp", "np", "np_cached", "tgs", "pgs", "scene", "persistent", "recip", "pyramid"]
    if "bp" in which:
        make_bp()
    if "np" in which:
        make_np()
    if "np_cached" in which:
        make_np_cached()
    if "tgs" in which:
        make_tgs()
    if "pgs" in which:
        make_pgs()
    if "scene" in which:
        make_scene()
    if "persistent" in which:
        make_persistent()
    if "recip" in which:
        make_recip()
    if "pyramid" in which:
        make_pyramid()
