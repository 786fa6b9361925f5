"""Seeded joint scenes for the 1D-constraint (joint) path: chains of boxes hung
from static anchors, each link joined to the previous one (or the anchor) by a
spherical, revolute, fixed, prismatic or sprung joint.  The joint rows
(Px1DConstraint, physx/include/PxConstraintDesc.h:194) are written here from
the current poses, standing in for a joint shader (the caller's solverPrep):
both the reference and the GB300 build receive the same rows, so only the
prep and solve differ between them.

Row conventions (the solver's, DyTGSContactPrep.cpp:2418): the constraint
velocity is J.v = linear0.vA + angular0.wA - linear1.vB - angular1.wB and a
row's geometric error E must change as dE/dt = J.v: an equality row's error
is axis.(anchorA - anchorB) (or the angle of frame A relative to frame B about
the axis), and a limit row's error is the distance to the limit, positive
while the limit holds (its impulse is one-sided, minImpulse 0).

Test infrastructure (fixtures and parity tests)."""
import numpy as np

# Px1DConstraint, 80 bytes
PX1D = np.dtype([("linear0", "<f4", 3), ("geometricError", "<f4"), ("angular0", "<f4", 3), ("velocityTarget", "<f4"),
                 ("linear1", "<f4", 3), ("minImpulse", "<f4"), ("angular1", "<f4", 3), ("maxImpulse", "<f4"),
                 ("mod0", "<f4"), ("mod1", "<f4"), ("flags", "<u2"), ("solveHint", "<u2"), ("pad", "<u4")])
assert PX1D.itemsize == 80

# Px1DConstraintFlag
SPRING, ACCELERATION_SPRING, RESTITUTION, KEEPBIAS, OUTPUT_FORCE, HAS_DRIVE_LIMIT, ANGULAR = 1, 2, 4, 8, 16, 32, 64
# PxConstraintSolveHint
NONE, EQUALITY, INEQUALITY = 0, 2048, 2049
# per-joint flags (params[16])
DISABLE_PREPROCESSING, IMPROVED_SLERP, DRIVE_LIMITS_ARE_FORCES = 1, 2, 4
PARAM_FLOATS = 20
KINDS = ("spherical", "revolute", "fixed", "prismatic", "sprung")
FLT_MAX = np.float32(3.4028234663852886e38)


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by + ay * bw + az * bx - ax * bz,
                     aw * bz + az * bw + ax * by - ay * bx, aw * bw - ax * bx - ay * by - az * bz], np.float64)


def _qconj(q):
    return np.array([-q[0], -q[1], -q[2], q[3]], np.float64)


def _qrot(q, v):
    u = np.asarray(q[:3], np.float64)
    w = float(q[3])
    v = np.asarray(v, np.float64)
    return 2.0 * np.dot(u, v) * u + (w * w - np.dot(u, u)) * v + 2.0 * w * np.cross(u, v)


def _qaxes(q):
    return [_qrot(q, e) for e in np.eye(3)]


def _random_quat(rng, scale):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = rng.uniform(-scale, scale)
    return np.concatenate([axis * np.sin(ang / 2), [np.cos(ang / 2)]])


def make_joint_scene(seed, nb_chains=6, links=(3, 8), kinds=KINDS):
    """Bodies (PxRigidBodyData), static anchors and per-joint description: the two
    bodies, local anchor frames, kind and settings."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from physx_gb300.workloads import rigid_body_data, mass_properties
    rng = np.random.default_rng(seed)
    counts = [int(rng.integers(links[0], links[1] + 1)) for _ in range(nb_chains)]
    n = sum(counts)
    rigid = rigid_body_data(n)
    statics = np.zeros((nb_chains, 7), np.float32)
    joints = []
    b = 0
    for c in range(nb_chains):
        top = np.array([4.0 * c, 12.0, 0.0])
        statics[c, :4] = [0, 0, 0, 1]
        statics[c, 4:] = top
        prev = n + c       # the anchor: a static body
        for k in range(counts[c]):
            half = rng.uniform(0.15, 0.45, size=3)
            inv_m, inv_i = mass_properties(3, half, density=float(rng.uniform(300.0, 1500.0)))
            centre = top - np.array([0.0, (2 * k + 1) * 0.55 + 0.1 * k, 0.0]) + rng.normal(scale=0.03, size=3)
            q = _random_quat(rng, 0.15)
            rigid[b]["invMass"] = inv_m
            rigid[b]["invInertia"] = inv_i
            rigid[b]["q"] = q.astype(np.float32)
            rigid[b]["p"] = centre.astype(np.float32)
            rigid[b]["linVel"] = rng.normal(scale=0.3, size=3).astype(np.float32)
            rigid[b]["angVel"] = rng.normal(scale=0.5, size=3).astype(np.float32)
            # joint point halfway between the two bodies (in world, at rest)
            pprev = top if prev >= n else rigid[prev]["p"].astype(np.float64)
            qprev = np.array([0, 0, 0, 1.0]) if prev >= n else rigid[prev]["q"].astype(np.float64)
            jp = 0.5 * (pprev + centre) + rng.normal(scale=0.02, size=3)
            jq = _random_quat(rng, 0.3)
            local0 = np.concatenate([_qmul(_qconj(qprev), jq), _qrot(_qconj(qprev), jp - pprev)])
            local1 = np.concatenate([_qmul(_qconj(q), jq), _qrot(_qconj(q), jp - centre)])
            kind = kinds[int(rng.integers(len(kinds)))]
            j = dict(a=prev, b=b, local0=local0, local1=local1, kind=kind,
                     scales=np.array([1.0, 1.0, 1.0, 1.0], np.float32), flags=0, lin_break=FLT_MAX, ang_break=FLT_MAX,
                     min_response=np.float32(0.0), limit=float(rng.uniform(0.05, 0.4)), stiffness=float(rng.uniform(50.0, 400.0)),
                     damping=float(rng.uniform(1.0, 20.0)), drive_vel=float(rng.uniform(-1.0, 1.0)),
                     drive_limit=float(rng.uniform(5.0, 50.0)), restitution=float(rng.uniform(0.0, 0.6)),
                     accel=bool(rng.integers(2)), output_force=bool(rng.integers(2)))
            u = rng.uniform()
            if u < 0.15:
                j["scales"] = np.array([rng.uniform(0.5, 1.5), rng.uniform(0.5, 1.5), rng.uniform(0.5, 1.5), rng.uniform(0.5, 1.5)], np.float32)
            elif u < 0.25:
                j["flags"] |= DISABLE_PREPROCESSING
            elif u < 0.35:
                j["lin_break"] = np.float32(rng.uniform(1.0, 30.0))
                j["ang_break"] = np.float32(rng.uniform(1.0, 30.0))
            if rng.uniform() < 0.4:
                j["flags"] |= DRIVE_LIMITS_ARE_FORCES
            joints.append(j)
            prev = b
            b += 1
    return dict(rigid=rigid, static_poses=statics, joints=joints, nb_dyn=n)


def _pose_of(scene, rigid, idx):
    n = scene["nb_dyn"]
    if idx >= n:
        s = scene["static_poses"][idx - n].astype(np.float64)
        return s[:4], s[4:]
    return rigid[idx]["q"].astype(np.float64), rigid[idx]["p"].astype(np.float64)


def joint_rows(scene, rigid):
    """Rows and per-joint parameters for the scene's joints at the poses in `rigid`:
    (rows PX1D array, rowStart, rowCount, params float32 (J, 20))."""
    rows = []
    start, count = [], []
    params = np.zeros((len(scene["joints"]), PARAM_FLOATS), np.float32)
    for ji, j in enumerate(scene["joints"]):
        qa, pa = _pose_of(scene, rigid, j["a"])
        qb, pb = _pose_of(scene, rigid, j["b"])
        la, lb = j["local0"], j["local1"]
        ca_q = _qmul(qa, la[:4])
        cb_q = _qmul(qb, lb[:4])
        ca_p = pa + _qrot(qa, la[4:])
        cb_p = pb + _qrot(qb, lb[4:])
        ra, rb = ca_p - pa, cb_p - pb
        axes = _qaxes(ca_q)
        d = cb_p - ca_p
        rel = _qmul(cb_q, _qconj(ca_q))
        if rel[3] < 0:
            rel = -rel
        rot = 2.0 * rel[:3]            # small-angle rotation of frame B relative to frame A, world
        jr = []

        def lin(axis, err, hint=EQUALITY, flags=0, lo=-FLT_MAX, hi=FLT_MAX, m0=0.0, m1=0.0, vt=0.0):
            r = np.zeros((), PX1D)
            r["linear0"], r["angular0"] = axis, np.cross(ra, axis)
            r["linear1"], r["angular1"] = axis, np.cross(rb, axis)
            r["geometricError"], r["velocityTarget"] = err, vt
            r["minImpulse"], r["maxImpulse"] = lo, hi
            r["mod0"], r["mod1"] = m0, m1
            r["flags"], r["solveHint"] = flags, hint
            jr.append(r)

        def ang(axis, err, hint=EQUALITY, flags=0, lo=-FLT_MAX, hi=FLT_MAX, m0=0.0, m1=0.0, vt=0.0):
            r = np.zeros((), PX1D)
            r["angular0"], r["angular1"] = axis, axis
            r["geometricError"], r["velocityTarget"] = err, vt
            r["minImpulse"], r["maxImpulse"] = lo, hi
            r["mod0"], r["mod1"] = m0, m1
            r["flags"], r["solveHint"] = flags | ANGULAR, hint
            jr.append(r)

        out = OUTPUT_FORCE if j["output_force"] else 0
        kind = j["kind"]
        if kind in ("spherical", "revolute", "fixed", "sprung"):
            for a in axes:
                lin(a, -np.dot(a, d), flags=out)
        if kind == "prismatic":
            for a in axes[1:]:
                lin(a, -np.dot(a, d), flags=out)
            # travel along x limited to +-limit, with restitution
            x = np.dot(axes[0], d)
            lin(axes[0], j["limit"] - x, hint=INEQUALITY, flags=out | RESTITUTION, lo=0.0, m0=j["restitution"], m1=0.2)
            lin(-axes[0], j["limit"] + x, hint=INEQUALITY, flags=out | RESTITUTION, lo=0.0, m0=j["restitution"], m1=0.2)
        if kind in ("revolute", "fixed", "prismatic"):
            free = 0 if kind == "revolute" else -1
            for i, a in enumerate(axes):
                if i != free:
                    ang(a, -np.dot(a, rot), flags=out)
        if kind == "revolute":
            # twist limit about the free axis, and a velocity drive with a force limit
            t = np.dot(axes[0], rot)
            ang(axes[0], j["limit"] - t, hint=INEQUALITY, flags=out | KEEPBIAS, lo=0.0)
            ang(axes[0], 0.0, hint=NONE, flags=out | SPRING | HAS_DRIVE_LIMIT, lo=-j["drive_limit"], hi=j["drive_limit"],
                m0=0.0, m1=j["damping"], vt=j["drive_vel"])
        if kind == "sprung":
            for a in axes:
                fl = out | SPRING | (ACCELERATION_SPRING if j["accel"] else 0) | HAS_DRIVE_LIMIT
                ang(a, -np.dot(a, rot), hint=NONE, flags=fl, lo=-j["drive_limit"], hi=j["drive_limit"], m0=j["stiffness"],
                    m1=j["damping"])
        start.append(len(rows))
        count.append(len(jr))
        rows.extend(jr)
        p = params[ji]
        p[0:4] = j["scales"]
        p[4:7] = ca_p
        p[7:10] = cb_p
        p[10:13] = 0.0
        p[13], p[14], p[15] = j["lin_break"], j["ang_break"], j["min_response"]
        p[16] = j["flags"]
    out_rows = np.zeros(len(rows), PX1D)
    for i, r in enumerate(rows):
        out_rows[i] = r
    return out_rows, np.array(start, np.uint32), np.array(count, np.uint32), params


def joint_arrays(scene):
    A = np.array([j["a"] for j in scene["joints"]], np.uint32)
    B = np.array([j["b"] for j in scene["joints"]], np.uint32)
    return A, B


def joint_frame(scene, rigid):
    """Everything one joint frame takes: bodies, anchors, the joints' bodies and
    their rows and parameters at the poses in `rigid`."""
    rows, rs, rc, pr = joint_rows(scene, rigid)
    A, B = joint_arrays(scene)
    return dict(nb_dyn=scene["nb_dyn"], static_poses=scene["static_poses"], joint_a=A, joint_b=B, rigid=rigid, rows=rows, row_start=rs,
                row_count=rc, params=pr)


def load_joint_fixture(path):
    """Frames of a joint fixture (tests/golden/make_joints.py): each a joint_frame
    dict plus the reference's outputs under ref_*."""
    import os, sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from physx_gb300.workloads import rigid_body_data
    z = np.load(path)
    rigid_dtype = rigid_body_data(0).dtype
    frames = []
    for f in z["frames"]:
        p = "f%d_" % f
        fr = dict(nb_dyn=int(z["nb_dyn"]), static_poses=z["static_poses"], joint_a=z["joint_a"], joint_b=z["joint_b"],
                  rigid=np.ascontiguousarray(z[p + "rigid"]).view(rigid_dtype).reshape(-1),
                  rows=np.ascontiguousarray(z[p + "rows"]).view(PX1D).reshape(-1), row_start=z[p + "row_start"], row_count=z[p + "row_count"],
                  params=z[p + "params"], frame=int(f))
        for k in ("vel", "pose", "header_start", "header_stride", "header_type", "order", "force", "broken"):
            fr["ref_" + k] = z[p + "ref_" + k]
        frames.append(fr)
    return frames
