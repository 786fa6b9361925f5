"""Seeded synthetic inputs shared by the golden-fixture generator and the tests.

Broadphase frames follow the broadphase-stress workload's shape (centres
uniform in a cube, log-normal half-extents, a random fraction of boxes moved
by N(0, sigma) each frame) plus edge cases the reference handles: touching
faces, +0/-0 coordinates, equal min-X keys, static/kinematic/dynamic groups,
shared (compound) group ids, per-object distances, removals and re-creations.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from physx_gb300.workloads import (batched_scenes, mass_properties, plane_pose_y_up, random_quat,  # noqa: E402,F401
                                  rigid_body_data)


def filter_group(kind, i):
    """PxGetBroadPhase{Static,Kinematic,Dynamic}FilterGroup (physx/include/PxBroadPhase.h:264-291)."""
    if kind == 0:
        return 0
    return ((i + 1) << 3) | (1 if kind == 1 else 2)


def bp_frames(seed, n, frames, extent=100.0, move_frac=0.1, sigma=0.2, mu=np.log(0.5), s=0.5, edge_cases=True,
              removals=True, distances=True):
    """Yields dicts with created/updated/removed/bounds/groups/distances/capacity per frame."""
    rng = np.random.default_rng(seed)
    cap = n
    centres = rng.uniform(0.0, extent, size=(n, 3)).astype(np.float32)
    half = np.exp(rng.normal(mu, s, size=(n, 3))).astype(np.float32)
    kinds = rng.choice([0, 1, 2], size=n, p=[0.1, 0.1, 0.8])
    ids = np.arange(n)
    if edge_cases:
        # compound actors: pairs of boxes share a dynamic id
        shared = rng.choice(n, size=max(2, n // 50), replace=False)
        ids[shared[1::2]] = ids[shared[0::2]][: len(shared[1::2])]
        kinds[shared] = 2
    groups = np.array([filter_group(k, i) for k, i in zip(kinds, ids)], dtype=np.uint32)
    dist = (rng.uniform(0.0, 0.05, size=n).astype(np.float32) if distances else np.zeros(n, np.float32))
    bounds = np.zeros((cap + 1, 6), np.float32)
    bounds[:n, :3] = centres - half
    bounds[:n, 3:] = centres + half
    if edge_cases and n >= 16:
        # exact touching faces along x, y, z and a -0/+0 pair, equal min-x keys
        bounds[0] = [0.0, 0.0, 0.0, 1.0, 1.0, 1.0]
        bounds[1] = [1.0, 0.0, 0.0, 2.0, 1.0, 1.0]
        bounds[2] = [0.0, 1.0, 0.0, 1.0, 2.0, 1.0]
        bounds[3] = [0.0, 0.0, 1.0, 1.0, 1.0, 2.0]
        bounds[4] = [-1.0, 5.0, 5.0, -0.0, 6.0, 6.0]
        bounds[5] = [0.0, 5.0, 5.0, 1.0, 6.0, 6.0]
        bounds[6] = [10.0, 10.0, 10.0, 11.0, 11.0, 11.0]
        bounds[7] = [10.0, 10.5, 10.5, 12.0, 12.0, 12.0]
        for k in range(8):
            kinds[k] = 2
            groups[k] = filter_group(2, 100000 + k)
        dist[:8] = 0.0
    live = np.ones(n, bool)
    yield dict(created=np.arange(n, dtype=np.uint32), updated=np.zeros(0, np.uint32), removed=np.zeros(0, np.uint32),
               bounds=bounds.copy(), groups=groups.copy(), distances=dist.copy(), capacity=cap)
    for f in range(1, frames):
        alive = np.flatnonzero(live)
        nmove = max(1, int(len(alive) * move_frac))
        moved = rng.choice(alive, size=nmove, replace=False)
        created = np.zeros(0, np.int64)
        removed = np.zeros(0, np.int64)
        if removals and len(alive) > 8:
            rem_pool = np.setdiff1d(alive, moved)
            rem_pool = rem_pool[rem_pool >= 8]
            if len(rem_pool):
                removed = rng.choice(rem_pool, size=max(1, len(alive) // 100), replace=False)
                live[removed] = False
            dead = np.flatnonzero(~live)
            dead = np.setdiff1d(dead, removed)
            if len(dead):
                created = rng.choice(dead, size=max(1, len(dead) // 2), replace=False)
                live[created] = True
        # displace the moved boxes (and some static ones too: the reference lets
        # the user update any object)
        disp = rng.normal(0.0, sigma, size=(len(moved), 3)).astype(np.float32)
        bounds[moved, :3] += disp
        bounds[moved, 3:] += disp
        if len(created):
            c = rng.uniform(0.0, extent, size=(len(created), 3)).astype(np.float32)
            h = np.exp(rng.normal(mu, s, size=(len(created), 3))).astype(np.float32)
            bounds[created, :3] = c - h
            bounds[created, 3:] = c + h
        if edge_cases and f == 1 and n >= 16:
            # move box 1 so it exactly touches box 0 again from the other side
            bounds[1] = [-1.0, 0.0, 0.0, 0.0, 1.0, 1.0]
            moved = np.union1d(moved, [1])
        yield dict(created=np.sort(created).astype(np.uint32), updated=np.sort(moved).astype(np.uint32),
                   removed=np.sort(removed).astype(np.uint32), bounds=bounds.copy(), groups=groups.copy(),
                   distances=dist.copy(), capacity=cap)


def sorted_pairs(a):
    """Canonical form of a pair list: (n, 2) uint32 with id0 < id1, lexicographically sorted."""
    a = np.asarray(a, dtype=np.uint32).reshape(-1, 2)
    if len(a) == 0:
        return a
    a = np.sort(a, axis=1)
    order = np.lexsort((a[:, 1], a[:, 0]))
    return a[order]




def shape_params(rng, t):
    g = np.zeros(4, np.float32)
    if t == 0:
        g[0] = rng.uniform(0.25, 1.0)
    elif t == 2:
        g[0] = rng.uniform(0.2, 0.5)
        g[1] = rng.uniform(0.25, 1.0)
    elif t == 3:
        g[:3] = rng.uniform(0.25, 1.0, size=3)
    return g


def bounding_radius(t, g):
    if t == 0:
        return g[0]
    if t == 2:
        return g[0] + g[1]
    if t == 3:
        return float(np.linalg.norm(g[:3]))
    return 0.0


def np_pairs(seed, n, types=None, spread=0.6, flat_frac=0.2):
    """Near-contact pairs of every primitive combination.  Returns dict of arrays in the
    harness layout.  `flat_frac` of the box pairs are axis-aligned stacks (face contacts)."""
    rng = np.random.default_rng(seed)
    combos = types or [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (0, 3), (3, 0), (1, 2), (2, 1), (1, 3), (3, 1), (2, 2),
                       (2, 3), (3, 2), (3, 3)]
    t0 = np.zeros(n, np.int32)
    t1 = np.zeros(n, np.int32)
    g0 = np.zeros((n, 4), np.float32)
    g1 = np.zeros((n, 4), np.float32)
    p0 = np.zeros((n, 7), np.float32)
    p1 = np.zeros((n, 7), np.float32)
    q = random_quat(rng, 2 * n)
    for i in range(n):
        a, b = combos[i % len(combos)]
        t0[i], t1[i] = a, b
        g0[i], g1[i] = shape_params(rng, a), shape_params(rng, b)
        c0 = rng.uniform(-5, 5, size=3).astype(np.float32)
        p0[i, :4], p0[i, 4:] = q[2 * i], c0
        p1[i, :4] = q[2 * i + 1]
        if a == 1 or b == 1:
            # plane at y = 0 (or tilted slightly); other shape near it
            pl = plane_pose_y_up()
            other = 1 if a == 1 else 0
            sh = g1[i] if other == 1 else g0[i]
            ts = b if other == 1 else a
            h = bounding_radius(ts, sh)
            pos = np.array([rng.uniform(-3, 3), rng.uniform(-0.3, 1.0) * h, rng.uniform(-3, 3)], np.float32)
            if a == 1:
                p0[i] = pl
                p1[i, 4:] = pos
            else:
                p1[i] = pl
                p0[i, 4:] = pos
            if rng.random() < flat_frac:
                (p1 if a == 1 else p0)[i, :4] = [0, 0, 0, 1]
            continue
        r0, r1 = bounding_radius(a, g0[i]), bounding_radius(b, g1[i])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        dist = (r0 + r1) * rng.uniform(0.35, 1.0 + spread * 0.1)
        p1[i, 4:] = c0 + (d * dist).astype(np.float32)
        if a == 3 and b == 3 and rng.random() < flat_frac:
            # stacked boxes: aligned, one above the other with a small yaw
            p0[i, :4] = [0, 0, 0, 1]
            yaw = rng.uniform(-0.05, 0.05)
            p1[i, :4] = [0, np.sin(yaw / 2), 0, np.cos(yaw / 2)]
            p1[i, 4:] = c0 + np.array([rng.uniform(-0.2, 0.2), g0[i, 1] + g1[i, 1] - rng.uniform(0.0, 0.03),
                                       rng.uniform(-0.2, 0.2)], np.float32)
    return dict(type0=t0, geom0=g0, type1=t1, geom1=g1, pose0=p0, pose1=p1)




def random_scene(seed, nbodies, spread=None, shapes=(0, 2, 3), drop=(0.2, 3.0), friction=(0.3, 0.8), plane=True,
                 jitter_vel=0.5):
    """A compact pile of random spheres/capsules/boxes above (and touching) a y=0 plane.
    Returns dict: types (n,), geoms (n,4), rigid (PxRigidBodyData), statics poses (m,7), static types/geoms."""
    rng = np.random.default_rng(seed)
    spread = spread if spread is not None else max(1.0, np.sqrt(nbodies) * 0.9)
    types = np.array([shapes[i % len(shapes)] for i in range(nbodies)], np.int32)
    rng.shuffle(types)
    geoms = np.stack([shape_params(rng, t) for t in types])
    rb = rigid_body_data(nbodies)
    q = random_quat(rng, nbodies)
    for i in range(nbodies):
        im, ii = mass_properties(types[i], geoms[i])
        rb[i]["invMass"] = im
        rb[i]["invInertia"] = ii
        rb[i]["q"] = q[i]
        h = bounding_radius(types[i], geoms[i])
        rb[i]["p"] = [rng.uniform(-spread, spread), rng.uniform(*drop) * h, rng.uniform(-spread, spread)]
        rb[i]["linVel"] = rng.normal(0, jitter_vel, 3)
        rb[i]["angVel"] = rng.normal(0, jitter_vel, 3)
    mats = rng.uniform(*friction, size=nbodies).astype(np.float32)
    statics = np.array([plane_pose_y_up()]) if plane else np.zeros((0, 7), np.float32)
    return dict(types=types, geoms=geoms.astype(np.float32), rigid=rb, friction=mats, static_poses=statics,
                static_types=np.ones(len(statics), np.int32), static_geoms=np.zeros((len(statics), 4), np.float32))



def pile_scenes(seed, nb_scenes, n, **kw):
    """Like batched_scenes but every scene is a compact pile already in contact (for parity tests)."""
    out = [random_scene(seed + k, n, **kw) for k in range(nb_scenes)]
    rb = np.concatenate([o["rigid"] for o in out])
    return dict(body_count=np.full(nb_scenes, n, np.uint32), static_count=np.ones(nb_scenes, np.uint32), rigid=rb,
                types=np.concatenate([o["types"] for o in out]), geoms=np.concatenate([o["geoms"] for o in out]),
                friction=np.concatenate([o["friction"] for o in out]), static_poses=np.tile(plane_pose_y_up(), (nb_scenes, 1)),
                static_types=np.ones(nb_scenes, np.int32), static_geoms=np.zeros((nb_scenes, 4), np.float32))


def hub_scene(nb_spheres=40, seed=0):
    """One wide box on the ground plane carrying `nb_spheres` separated spheres: the
    box takes part in more than 32 dynamic constraints, so the batching needs a
    second round of 32 partitions, and the plane adds a static constraint."""
    from physx_gb300.workloads import mass_properties_batch, plane_pose_y_up, rigid_body_data
    rng = np.random.default_rng(seed)
    n = 1 + nb_spheres
    types = np.array([3] + [0] * nb_spheres, np.int32)
    geoms = np.zeros((n, 4), np.float32)
    geoms[0, :3] = (5.0, 0.5, 5.0)
    geoms[1:, 0] = 0.3
    rb = rigid_body_data(n)
    rb["p"][0] = (0.0, 0.49, 0.0)
    k = np.arange(nb_spheres)
    rb["p"][1:, 0] = (k % 7) * 1.2 - 3.6 + rng.uniform(-0.05, 0.05, nb_spheres)
    rb["p"][1:, 2] = (k // 7) * 1.2 - 3.6 + rng.uniform(-0.05, 0.05, nb_spheres)
    rb["p"][1:, 1] = 0.99 + 0.28 + rng.uniform(-0.01, 0.01, nb_spheres)
    im, ii = mass_properties_batch(types, geoms)
    rb["invMass"] = im
    rb["invInertia"] = ii
    return dict(body_count=np.array([n], np.uint32), static_count=np.ones(1, np.uint32), rigid=rb, types=types, geoms=geoms,
                friction=np.full(n, 0.5, np.float32), static_poses=plane_pose_y_up()[None, :].copy(), static_types=np.ones(1, np.int32),
                static_geoms=np.zeros((1, 4), np.float32))


def _quat_mul(a, b):
    ax, ay, az, aw = a.T
    bx, by, bz, bw = b.T
    return np.stack([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz], 1)


def perturb_poses(rng, pose, lin, ang):
    """Moves every pose by N(0, lin) m per axis and turns it by N(0, ang) rad about a random axis."""
    n = len(pose)
    out = pose.copy()
    out[:, 4:] += rng.normal(0, lin, size=(n, 3)).astype(np.float32)
    axis = rng.normal(size=(n, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    th = rng.normal(0, ang, size=n)
    dq = np.concatenate([axis * np.sin(th / 2)[:, None], np.cos(th / 2)[:, None]], 1)
    q = _quat_mul(dq, out[:, :4].astype(np.float64))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    out[:, :4] = q.astype(np.float32)
    return out


CACHED_KINDS = [(1, 2), (2, 1), (1, 3), (3, 1), (2, 3), (3, 2), (3, 3)]


def moving_pairs(seed, n, frames, types=None):
    """Near-contact pairs of the kinds whose contact manifold persists between frames
    (plane-capsule, plane-box, capsule-box, box-box), then `frames - 1` small motions:
    one body of every pair moves ~2 mm / 0.3 deg per frame, every fourth frame ~2 cm /
    3 deg (enough to invalidate a manifold).  Returns the pair dict of frame 0 and the
    (pose0, pose1) of every frame."""
    pairs = np_pairs(seed, n, types=types or CACHED_KINDS)
    rng = np.random.default_rng(seed + 1000)
    poses = [(pairs["pose0"].copy(), pairs["pose1"].copy())]
    for f in range(1, frames):
        p0, p1 = poses[-1]
        big = f % 4 == 0
        lin, ang = (0.02, 0.05) if big else (0.002, 0.005)
        if f % 2:
            p1 = perturb_poses(rng, p1, lin, ang)
        else:
            p0 = perturb_poses(rng, p0, lin, ang)
        poses.append((p0, p1))
    return pairs, poses
