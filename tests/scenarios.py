"""Seeded synthetic inputs shared by the golden-fixture generator and the tests.

Broadphase frames follow the broadphase-stress workload's shape (centres
uniform in a cube, log-normal half-extents, a random fraction of boxes moved
by N(0, sigma) each frame) plus edge cases the reference handles: touching
faces, +0/-0 coordinates, equal min-X keys, static/kinematic/dynamic groups,
shared (compound) group ids, per-object distances, removals and re-creations.
"""
import numpy as np


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


def random_quat(rng, n):
    """Haar-uniform unit quaternions (Shoemake), (n, 4) as (x, y, z, w)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    return q.astype(np.float32)


def plane_pose_y_up():
    """PxTransformFromPlaneEquation(PxPlane(0,1,0,0)): x axis of the plane frame -> +y."""
    s = np.float32(np.sqrt(0.5))
    return np.array([0.0, 0.0, s, s, 0.0, 0.0, 0.0], np.float32)


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


def rigid_body_data(n):
    """Zeroed PxRigidBodyData array (physx/include/PxImmediateMode.h:68), 96 bytes each,
    with the reference's rigid-dynamic defaults (ScBodyCore.cpp:50-54, PxvDynamics.h:140)."""
    dt = np.dtype([("linVel", "<f4", 3), ("invMass", "<f4"), ("angVel", "<f4", 3), ("maxDepenetrationVelocity", "<f4"),
                   ("invInertia", "<f4", 3), ("maxContactImpulse", "<f4"), ("q", "<f4", 4), ("p", "<f4", 3),
                   ("linearDamping", "<f4"), ("angularDamping", "<f4"), ("maxLinearVelocitySq", "<f4"),
                   ("maxAngularVelocitySq", "<f4"), ("pad", "<u4")])
    assert dt.itemsize == 96
    r = np.zeros(n, dt)
    r["q"][:, 3] = 1.0
    r["maxDepenetrationVelocity"] = 1e32
    r["maxContactImpulse"] = 1e32
    r["linearDamping"] = 0.0
    r["angularDamping"] = 0.05
    r["maxLinearVelocitySq"] = 1e32
    r["maxAngularVelocitySq"] = 100.0 * 100.0
    return r


def mass_properties(t, g, density=1000.0):
    """Mass and mass-space inverse inertia diagonal of a sphere / capsule (along x) / box."""
    if t == 0:
        r = g[0]
        m = density * 4.0 / 3.0 * np.pi * r ** 3
        i = np.full(3, 0.4 * m * r * r)
    elif t == 3:
        hx, hy, hz = g[:3]
        m = density * 8.0 * hx * hy * hz
        i = np.array([m / 3.0 * (hy * hy + hz * hz), m / 3.0 * (hx * hx + hz * hz), m / 3.0 * (hx * hx + hy * hy)])
    else:
        r, hh = g[0], g[1]
        mc = density * np.pi * r * r * 2.0 * hh       # cylinder
        ms = density * 4.0 / 3.0 * np.pi * r ** 3      # two hemispheres
        m = mc + ms
        ix = mc * r * r / 2.0 + ms * 0.4 * r * r
        iyz = mc * (r * r / 4.0 + (2 * hh) ** 2 / 12.0) + ms * (0.4 * r * r + hh * hh + 0.75 * hh * r)
        i = np.array([ix, iyz, iyz])
    return np.float32(1.0 / m), (1.0 / i).astype(np.float32)


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
