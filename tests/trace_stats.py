"""Physical statistics of a simulation trace, for long-horizon checks where
chaotic divergence makes per-body comparison meaningless: kinetic energy,
ground clearance (how far the lowest point of every body is above the plane
y = 0; negative = penetration), mean and top body heights, fraction of bodies
at rest.  Test infrastructure."""
import numpy as np

from physx_gb300.workloads import kinetic_energy

FIELDS = ("ke", "min_clearance", "mean_height", "top_height", "resting")


def _rotate(q, v):
    """Rotates vectors v (n, 3) by unit quaternions q (n, 4) as (x, y, z, w)."""
    qv, qw = q[:, :3], q[:, 3:4]
    t = 2.0 * np.cross(qv, v)
    return v + qw * t + np.cross(qv, t)


def ground_clearance(rigid, types, geoms):
    """Height of the lowest point of each body above y = 0: spheres p.y - r,
    capsules (axis along local x) p.y - |axis.y| hh - r, boxes p.y - sum_k |R_yk| h_k."""
    q = rigid["q"].astype(np.float64)
    p = rigid["p"].astype(np.float64)
    g = np.asarray(geoms, np.float64)
    n = len(types)
    ext = np.zeros(n)
    sph, cap, box = types == 0, types == 2, types == 3
    ext[sph] = g[sph, 0]
    if cap.any():
        ax = _rotate(q[cap], np.tile([1.0, 0.0, 0.0], (int(cap.sum()), 1)))
        ext[cap] = np.abs(ax[:, 1]) * g[cap, 1] + g[cap, 0]
    if box.any():
        nb = int(box.sum())
        for k in range(3):
            e = np.zeros((nb, 3))
            e[:, k] = 1.0
            ext[box] += np.abs(_rotate(q[box], e)[:, 1]) * g[box, k]
    return p[:, 1] - ext


def step_stats(rigid, types, geoms, rest_speed=0.05):
    v = np.linalg.norm(rigid["linVel"].astype(np.float64), axis=1)
    y = rigid["p"][:, 1].astype(np.float64)
    return dict(ke=kinetic_energy(rigid), min_clearance=float(ground_clearance(rigid, types, geoms).min()), mean_height=float(y.mean()),
                top_height=float(y.max()), resting=float((v < rest_speed).mean()))


def body_checksum(rigid):
    """A checksum of a body array's bytes (to confirm two machines start from the same state)."""
    b = np.frombuffer(np.ascontiguousarray(rigid).tobytes(), np.uint32)
    return int((b.astype(np.uint64) * (np.arange(len(b), dtype=np.uint64) % 65521 + 1)).sum() % (1 << 61))
