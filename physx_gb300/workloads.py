"""Synthetic workloads of the rigid-body step (seeded, no external data).

batched_scenes() is the batched workload: independent scenes with body counts
log-uniform in [8, 512] (sphere / box / capsule mix), dropped from U(1, 20) m
onto a per-scene ground plane.  Rigid bodies are PxRigidBodyData records
(physx/include/PxImmediateMode.h:68) with the reference's rigid-dynamic
defaults (physx/source/simulationcontroller/src/ScBodyCore.cpp:50-54).
"""
import numpy as np

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

def batched_scenes(seed, nb_scenes, nmin=8, nmax=512, shapes=(0, 2, 3), drop=(1.0, 20.0), friction=(0.3, 0.8)):
    """Independent scenes (the batched workload's shape): body counts log-uniform in
    [nmin, nmax], sphere/box/capsule mix, drop heights U(drop) m above a per-scene
    plane y=0, xz spread U(-sqrt(N), sqrt(N)) m, random orientations, zero velocity."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), nb_scenes)).astype(np.int64)
    counts = np.clip(counts, nmin, nmax).astype(np.uint32)
    N = int(counts.sum())
    types = rng.choice(np.array(shapes, np.int32), size=N)
    geoms = np.zeros((N, 4), np.float32)
    r = rng.uniform(0.25, 1.0, N)
    geoms[types == 0, 0] = r[types == 0]
    geoms[types == 3, :3] = rng.uniform(0.25, 1.0, (int((types == 3).sum()), 3))
    cap = types == 2
    geoms[cap, 0] = rng.uniform(0.2, 0.5, int(cap.sum()))
    geoms[cap, 1] = rng.uniform(0.25, 1.0, int(cap.sum()))
    rb = rigid_body_data(N)
    rb["q"] = random_quat(rng, N)
    spread = np.repeat(np.sqrt(counts.astype(np.float64)), counts)
    rb["p"][:, 0] = rng.uniform(-1, 1, N) * spread
    rb["p"][:, 2] = rng.uniform(-1, 1, N) * spread
    rb["p"][:, 1] = rng.uniform(drop[0], drop[1], N)
    im, ii = mass_properties_batch(types, geoms)
    rb["invMass"] = im
    rb["invInertia"] = ii
    fr = rng.uniform(friction[0], friction[1], N).astype(np.float32)
    S = nb_scenes
    return dict(body_count=counts, static_count=np.ones(S, np.uint32), rigid=rb, types=types.astype(np.int32), geoms=geoms,
                friction=fr, static_poses=np.tile(plane_pose_y_up(), (S, 1)), static_types=np.ones(S, np.int32),
                static_geoms=np.zeros((S, 4), np.float32))


def large_scene(seed=2, n=100_000, extent=100.0, height=200.0, friction=(0.3, 0.8)):
    """Single large scene: n bodies, 1/3 spheres r ~ U(0.25, 1), 1/3 boxes with
    half-extents ~ U(0.25, 1) per axis, 1/3 capsules r ~ U(0.2, 0.5), half-height
    ~ U(0.25, 1); positions U([-extent, extent] x [0, height] x [-extent, extent]),
    Haar-uniform orientations, zero velocity, friction U(friction), density 1000,
    on the plane y = 0.  Initial overlaps are allowed."""
    rng = np.random.default_rng(seed)
    types = np.array([0, 3, 2], np.int32)[np.arange(n) % 3]
    rng.shuffle(types)
    geoms = np.zeros((n, 4), np.float32)
    sph, box, cap = types == 0, types == 3, types == 2
    geoms[sph, 0] = rng.uniform(0.25, 1.0, int(sph.sum()))
    geoms[box, :3] = rng.uniform(0.25, 1.0, (int(box.sum()), 3))
    geoms[cap, 0] = rng.uniform(0.2, 0.5, int(cap.sum()))
    geoms[cap, 1] = rng.uniform(0.25, 1.0, int(cap.sum()))
    rb = rigid_body_data(n)
    rb["q"] = random_quat(rng, n)
    rb["p"][:, 0] = rng.uniform(-extent, extent, n)
    rb["p"][:, 1] = rng.uniform(0.0, height, n)
    rb["p"][:, 2] = rng.uniform(-extent, extent, n)
    im, ii = mass_properties_batch(types, geoms)
    rb["invMass"] = im
    rb["invInertia"] = ii
    fr = rng.uniform(friction[0], friction[1], n).astype(np.float32)
    return dict(rigid=rb, types=types, geoms=geoms, friction=fr, static_poses=np.array([plane_pose_y_up()], np.float32),
                static_types=np.ones(1, np.int32), static_geoms=np.zeros((1, 4), np.float32))


def as_world(scene):
    """One scene's arrays as a one-scene world (body_count / static_count added)."""
    return dict(scene, body_count=np.array([len(scene["types"])], np.uint32),
                static_count=np.array([len(scene["static_types"])], np.uint32))


def mass_properties_batch(types, geoms, density=1000.0):
    """Vectorised mass_properties: (invMass (n,), invInertia (n, 3))."""
    g = geoms.astype(np.float64)
    m = np.zeros(len(types))
    inertia = np.zeros((len(types), 3))
    sph = types == 0
    r = g[sph, 0]
    m[sph] = density * 4.0 / 3.0 * np.pi * r ** 3
    inertia[sph] = (0.4 * m[sph] * r * r)[:, None]
    box = types == 3
    hx, hy, hz = g[box, 0], g[box, 1], g[box, 2]
    m[box] = density * 8.0 * hx * hy * hz
    inertia[box] = np.stack([m[box] / 3.0 * (hy * hy + hz * hz), m[box] / 3.0 * (hx * hx + hz * hz), m[box] / 3.0 * (hx * hx + hy * hy)], 1)
    cap = types == 2
    r, hh = g[cap, 0], g[cap, 1]
    mc = density * np.pi * r * r * 2.0 * hh
    ms = density * 4.0 / 3.0 * np.pi * r ** 3
    m[cap] = mc + ms
    ix = mc * r * r / 2.0 + ms * 0.4 * r * r
    iyz = mc * (r * r / 4.0 + (2 * hh) ** 2 / 12.0) + ms * (0.4 * r * r + hh * hh + 0.75 * hh * r)
    inertia[cap] = np.stack([ix, iyz, iyz], 1)
    return (1.0 / m).astype(np.float32), (1.0 / inertia).astype(np.float32)


def pyramid_scene(seed=1, levels=20, half=0.5, density=1000.0, friction=0.5, jitter=0.01, yaw_deg=2.0):
    """The box pyramid of the reference's immediate-mode snippet
    (physx/snippets/snippetimmediatemode/SnippetImmediateMode.cpp:283-298):
    `levels` rows of unit boxes (half extent `half`), row i holding levels - i
    boxes at x = (2j - (levels - i)) * half, y = (2i + 1) * half, z = 0, each
    jittered by U(-jitter, jitter) m in x and z and U(-yaw, yaw) degrees about y;
    one static plane y = 0.  Returns one scene in the world layout."""
    rng = np.random.default_rng(seed)
    pos = []
    for i in range(levels):
        for j in range(levels - i):
            pos.append(((2 * j - (levels - i)) * half, (2 * i + 1) * half, 0.0))
    n = len(pos)
    pos = np.array(pos, np.float64)
    pos[:, 0] += rng.uniform(-jitter, jitter, n)
    pos[:, 2] += rng.uniform(-jitter, jitter, n)
    yaw = np.radians(rng.uniform(-yaw_deg, yaw_deg, n))
    rb = rigid_body_data(n)
    rb["p"] = pos.astype(np.float32)
    rb["q"] = np.stack([np.zeros(n), np.sin(yaw / 2), np.zeros(n), np.cos(yaw / 2)], 1).astype(np.float32)
    types = np.full(n, 3, np.int32)
    geoms = np.zeros((n, 4), np.float32)
    geoms[:, :3] = half
    im, ii = mass_properties_batch(types, geoms, density)
    rb["invMass"] = im
    rb["invInertia"] = ii
    return dict(body_count=np.array([n], np.uint32), static_count=np.ones(1, np.uint32), rigid=rb, types=types, geoms=geoms,
                friction=np.full(n, friction, np.float32), static_poses=plane_pose_y_up()[None, :].copy(),
                static_types=np.ones(1, np.int32), static_geoms=np.zeros((1, 4), np.float32))


def kinetic_energy(rigid):
    """Translational + rotational kinetic energy of PxRigidBodyData records (mass-space
    inertia, world angular velocity rotated into the body frame)."""
    m = 1.0 / rigid["invMass"].astype(np.float64)
    v = rigid["linVel"].astype(np.float64)
    w = rigid["angVel"].astype(np.float64)
    q = rigid["q"].astype(np.float64)
    # rotate w into the body frame: q^-1 * w
    qv, qw = -q[:, :3], q[:, 3:4]
    t = 2.0 * np.cross(qv, w)
    wl = w + qw * t + np.cross(qv, t)
    inertia = 1.0 / rigid["invInertia"].astype(np.float64)
    return float(0.5 * (m * (v * v).sum(1)).sum() + 0.5 * (inertia * wl * wl).sum())


def aabb_stress_frames(seed=3, n=1_000_000, frames=10, extent=1000.0, move_frac=0.1, sigma=0.2):
    """Broadphase stress workload: n AABBs, centres U(0, extent)^3, per-axis
    half-extents lognormal(ln 0.5, 0.5), every box dynamic with its own filter
    group (PxGetBroadPhaseDynamicFilterGroup(i)), distance 0.  The first frame
    creates every box; each later frame moves move_frac of them (chosen without
    replacement) by N(0, sigma) m per axis and submits them as updated.  Yields
    dicts of created / updated / removed / bounds / groups / distances / capacity
    (bounds hold capacity + 1 rows, PxBounds3 layout)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, extent, size=(n, 3)).astype(np.float32)
    half = np.exp(rng.normal(np.log(0.5), 0.5, size=(n, 3))).astype(np.float32)
    bounds = np.zeros((n + 1, 6), np.float32)
    bounds[:n, :3] = centres - half
    bounds[:n, 3:] = centres + half
    groups = ((np.arange(n, dtype=np.uint32) + 1) << 3) | 2
    dist = np.zeros(n, np.float32)
    empty = np.zeros(0, np.uint32)
    yield dict(created=np.arange(n, dtype=np.uint32), updated=empty, removed=empty, bounds=bounds, groups=groups, distances=dist, capacity=n)
    m = max(1, int(n * move_frac))
    for _ in range(1, frames):
        moved = rng.choice(n, size=m, replace=False).astype(np.uint32)
        d = rng.normal(0.0, sigma, size=(m, 3)).astype(np.float32)
        bounds[moved, :3] += d
        bounds[moved, 3:] += d
        yield dict(created=empty, updated=np.sort(moved), removed=empty, bounds=bounds, groups=groups, distances=dist, capacity=n)


CONVEX_CORE = 4   # PxGeometryType::eCONVEXCORE
CORE_NAMES = ("point", "segment", "box", "ellipsoid", "cylinder", "cone")   # PxConvexCore::Type


def convex_core_type(core):
    """The shape type of a PxConvexCoreGeometry in the narrowphase's encoding:
    PxGeometryType 4 in the low byte, the PxConvexCore::Type in bits 8..15."""
    return CONVEX_CORE | (int(core) << 8)


def convex_core_params(rng, core):
    """Core floats and margin (4 floats) of a random convex core of the given type,
    with flat / degenerate variants (zero-margin boxes, disk and needle
    ellipsoids, flat cylinders) in the mix."""
    g = np.zeros(4, np.float32)
    if core == 0:
        g[3] = rng.uniform(0.15, 0.6)
    elif core == 1:
        g[0] = rng.uniform(0.2, 1.5)
        g[3] = rng.uniform(0.05, 0.3)
    elif core == 2:
        g[:3] = rng.uniform(0.2, 1.5, size=3)
        if rng.random() < 0.1:
            g[rng.integers(3)] = 0.0          # a flat box (a rectangle grown by the margin)
        g[3] = 0.0 if rng.random() < 0.4 else rng.uniform(0.01, 0.1)
    elif core == 3:
        g[:3] = rng.uniform(0.1, 0.8, size=3)
        u = rng.random()
        if u < 0.15:
            g[rng.integers(3)] = 0.0          # a disk
        elif u < 0.25:
            keep = rng.integers(3)
            g[[k for k in range(3) if k != keep]] = 0.0   # a needle
        g[3] = 0.0 if rng.random() < 0.5 else rng.uniform(0.01, 0.05)
    else:
        g[0] = rng.uniform(0.2, 1.5) if rng.random() > 0.1 else 0.0
        g[1] = rng.uniform(0.1, 0.6)
        g[3] = 0.0 if rng.random() < 0.5 else rng.uniform(0.01, 0.05)
    return g


def convex_core_radius(core, g):
    """Radius of a sphere about the shape's origin that holds the convex core."""
    if core == 0:
        r = 0.0
    elif core == 1:
        r = 0.5 * g[0]
    elif core == 2:
        r = 0.5 * float(np.linalg.norm(g[:3]))
    elif core == 3:
        r = float(g[:3].max())
    else:
        r = float(np.hypot(0.5 * g[0], g[1]))
    return r + float(g[3])


def _axis_aligned_quat(rng, jitter):
    """One of the 24 rotations that map axes to axes, turned by up to `jitter` radians."""
    base = [np.array([0, 0, 0, 1.0]), np.array([1.0, 0, 0, 0]), np.array([0, 1.0, 0, 0]), np.array([0, 0, 1.0, 0])]
    h = np.sqrt(0.5)
    base += [np.array(v) for v in ([h, 0, 0, h], [0, h, 0, h], [0, 0, h, h], [-h, 0, 0, h], [0, -h, 0, h], [0, 0, -h, h])]
    q = base[rng.integers(len(base))]
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    a = rng.uniform(-jitter, jitter)
    d = np.concatenate([ax * np.sin(a / 2), [np.cos(a / 2)]])
    # quaternion product d * q, (x, y, z, w)
    x1, y1, z1, w1 = d
    x2, y2, z2, w2 = q
    r = np.array([w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2, w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
                  w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2, w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2])
    return (r / np.linalg.norm(r)).astype(np.float32)


def convex_core_pairs(seed, n, aligned_frac=0.4):
    """Near-contact pairs with at least one convex core (PxConvexCoreGeometry of
    every core type) against spheres, planes, capsules, boxes and other convex
    cores, in both argument orders.  `aligned_frac` of the pairs have axis-aligned
    orientations (within 0.02 rad) and are offset along an axis, so that the
    contact faces of the cores (and the face clipping) are exercised.  Returns
    the narrowphase's pair arrays (type0, geom0, type1, geom1, pose0, pose1)."""
    rng = np.random.default_rng(seed)
    t0 = np.zeros(n, np.int32)
    t1 = np.zeros(n, np.int32)
    g0 = np.zeros((n, 4), np.float32)
    g1 = np.zeros((n, 4), np.float32)
    p0 = np.zeros((n, 7), np.float32)
    p1 = np.zeros((n, 7), np.float32)
    prim = {0: lambda: np.array([rng.uniform(0.25, 1.0), 0, 0, 0], np.float32),
            2: lambda: np.array([rng.uniform(0.2, 0.5), rng.uniform(0.25, 1.0), 0, 0], np.float32),
            3: lambda: np.concatenate([rng.uniform(0.25, 1.0, size=3), [0]]).astype(np.float32)}
    prim_radius = {0: lambda g: g[0], 2: lambda g: g[0] + g[1], 3: lambda g: float(np.linalg.norm(g[:3]))}
    for i in range(n):
        core = int(rng.integers(6))
        tc, gc, rc = convex_core_type(core), convex_core_params(rng, core), 0.0
        rc = convex_core_radius(core, gc)
        other = int(rng.integers(5))   # 0 sphere, 1 plane, 2 capsule, 3 box, 4 another convex core
        if other == 4:
            core2 = int(rng.integers(6))
            to, go = convex_core_type(core2), convex_core_params(rng, core2)
            ro = convex_core_radius(core2, go)
        elif other == 1:
            to, go, ro = 1, np.zeros(4, np.float32), 0.0
        else:
            to = other
            go = prim[other]()
            ro = prim_radius[other](go)
        aligned = rng.random() < aligned_frac
        qc = _axis_aligned_quat(rng, 0.02) if aligned else random_quat(rng, 1)[0]
        qo = _axis_aligned_quat(rng, 0.02) if aligned else random_quat(rng, 1)[0]
        c0 = rng.uniform(-5, 5, size=3).astype(np.float32)
        if other == 1:
            po = plane_pose_y_up()
            po[4:] = [rng.uniform(-3, 3), 0.0, rng.uniform(-3, 3)]
            pc = np.concatenate([qc, [po[4] + rng.uniform(-1, 1), rng.uniform(-0.3, 1.0) * rc, po[6] + rng.uniform(-1, 1)]])
        else:
            if aligned:
                d = np.zeros(3)
                d[rng.integers(3)] = rng.choice([-1.0, 1.0])
                d += rng.normal(size=3) * 0.05
            else:
                d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            dist = (rc + ro) * rng.uniform(0.4, 1.05)
            pc = np.concatenate([qc, c0])
            po = np.concatenate([qo, c0 + (d * dist).astype(np.float32)])
        first_core = rng.random() < 0.5
        if first_core:
            t0[i], g0[i], p0[i], t1[i], g1[i], p1[i] = tc, gc, pc, to, go, po
        else:
            t0[i], g0[i], p0[i], t1[i], g1[i], p1[i] = to, go, po, tc, gc, pc
    return dict(type0=t0, geom0=g0, type1=t1, geom1=g1, pose0=p0.astype(np.float32), pose1=p1.astype(np.float32))
