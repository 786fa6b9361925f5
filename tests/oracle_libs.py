"""ctypes loaders for the CPU oracle (oracle/liboracle.so) and, on the
development machine only, the reference built from source
(oracle/_ref/libpxref.so).  Test infrastructure: the GB300 package never
imports this module."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libpxref.so")

_oracle = None
_ref = None


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def oracle():
    global _oracle
    if _oracle is None:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        _oracle = ctypes.CDLL(ORACLE_SO)
        _oracle.orc_bp_create.restype = ctypes.c_void_p
        _oracle.orc_bp_release.argtypes = [ctypes.c_void_p]
    return _oracle


def reference():
    """The reference library, or None where it was not built (GPU machines)."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        _ref = ctypes.CDLL(REF_SO)
        _ref.pxref_bp_create.restype = ctypes.c_void_p
        _ref.pxref_bp_release.argtypes = [ctypes.c_void_p]
    return _ref


class CpuBroadPhase:
    """Same call pattern for the oracle ("orc") and the reference ("pxref")."""

    def __init__(self, which="orc", discard_sk=0, discard_kk=0, pabp=False):
        """pabp: the reference's ePABP broadphase instead of eABP (reference only)."""
        self.L = oracle() if which == "orc" else reference()
        self.pre = which
        if pabp:
            assert which == "pxref"
            self.L.pxref_bp_create_typed.restype = ctypes.c_void_p
            self.h = ctypes.c_void_p(self.L.pxref_bp_create_typed(1, discard_sk, discard_kk))
        else:
            self.h = ctypes.c_void_p(getattr(self.L, self.pre + "_bp_create")(discard_sk, discard_kk))

    def update(self, fr):
        cap = int(fr["capacity"])
        bounds = np.ascontiguousarray(fr["bounds"], np.float32)
        maxp = 1 << 20
        oc = np.zeros(2 * maxp, np.uint32)
        ol = np.zeros(2 * maxp, np.uint32)
        nc = np.zeros(1, np.uint32)
        nl = np.zeros(1, np.uint32)
        c = np.ascontiguousarray(fr["created"], np.uint32)
        u = np.ascontiguousarray(fr["updated"], np.uint32)
        r = np.ascontiguousarray(fr["removed"], np.uint32)
        g = np.ascontiguousarray(fr["groups"], np.uint32)
        d = np.ascontiguousarray(fr["distances"], np.float32)
        rc = getattr(self.L, self.pre + "_bp_update")(self.h, _p(c), len(c), _p(u), len(u), _p(r), len(r), _p(bounds), _p(g),
                                                      _p(d), cap, _p(oc), maxp, _p(nc), _p(ol), maxp, _p(nl))
        assert rc == 0, "pair buffer overflow"
        return oc[: 2 * nc[0]].reshape(-1, 2).copy(), ol[: 2 * nl[0]].reshape(-1, 2).copy()

    def release(self):
        if self.h:
            getattr(self.L, self.pre + "_bp_release")(self.h)
            self.h = None


def run_contacts(which, pairs, contact_distance=0.04, mesh_margin=0.01, tolerance_length=1.0, max_per_pair=16):
    """PxGenerateContacts with fresh caches: returns (counts, contacts[n, max, 8])."""
    n = len(pairs["type0"])
    out = np.zeros((n, max_per_pair, 8), np.float32)
    cnt = np.zeros(n, np.uint32)
    args = [_p(np.ascontiguousarray(pairs[k])) for k in ("type0", "geom0", "type1", "geom1", "pose0", "pose1")]
    if which == "orc":
        L = oracle()
        rc = L.orc_np_run(*args, ctypes.c_uint32(n), ctypes.c_float(contact_distance), ctypes.c_float(mesh_margin),
                          ctypes.c_float(tolerance_length), _p(out), ctypes.c_uint32(max_per_pair), _p(cnt))
    else:
        L = reference()
        L.pxref_np_create.restype = ctypes.c_void_p
        ctx = ctypes.c_void_p(L.pxref_np_create(ctypes.c_uint32(n)))
        rc = L.pxref_np_run(ctx, *args, ctypes.c_uint32(n), ctypes.c_float(contact_distance), ctypes.c_float(mesh_margin),
                            ctypes.c_float(tolerance_length), 1, _p(out), ctypes.c_uint32(max_per_pair), _p(cnt))
        L.pxref_np_release(ctx)
    assert rc == 0, "contact buffer overflow"
    return cnt, out


def scene_pairs(scene):
    """All dynamic-dynamic pairs (i < j) and every dynamic body against every static
    shape, in that order: (bodyA, bodyB) with statics indexed after the dynamics."""
    n = len(scene["types"])
    m = len(scene["static_poses"])
    A, B = [], []
    for i in range(n):
        for j in range(i + 1, n):
            A.append(i)
            B.append(j)
        for s in range(m):
            A.append(i)
            B.append(n + s)
    return np.array(A, np.uint32), np.array(B, np.uint32)


def scene_contacts(which, scene, A, B, contact_distance=0.04):
    """Fresh-cache contacts for the given pairs (through `which` narrowphase);
    returns per-pair (start, count) into a packed contact array plus the pair materials."""
    n = len(scene["types"])
    rb = scene["rigid"]

    def pose_of(k):
        if k < n:
            return np.concatenate([rb[k]["q"], rb[k]["p"]]).astype(np.float32)
        return scene["static_poses"][k - n]

    def geom_of(k):
        return (scene["types"][k], scene["geoms"][k]) if k < n else (scene["static_types"][k - n], scene["static_geoms"][k - n])

    pairs = dict(type0=np.array([geom_of(a)[0] for a in A], np.int32), geom0=np.array([geom_of(a)[1] for a in A], np.float32),
                 type1=np.array([geom_of(b)[0] for b in B], np.int32), geom1=np.array([geom_of(b)[1] for b in B], np.float32),
                 pose0=np.array([pose_of(a) for a in A], np.float32), pose1=np.array([pose_of(b) for b in B], np.float32))
    cnt, out = run_contacts(which, pairs, contact_distance=contact_distance)
    keep = np.flatnonzero(cnt > 0)
    start = np.zeros(len(keep), np.uint32)
    count = cnt[keep].astype(np.uint32)
    start[1:] = np.cumsum(count)[:-1]
    packed = np.concatenate([out[k, :cnt[k]] for k in keep]) if len(keep) else np.zeros((0, 8), np.float32)
    fr = scene["friction"]
    mat = np.zeros((len(keep), 3), np.float32)
    for r, k in enumerate(keep):
        fa = fr[A[k]]
        fb = fr[B[k]] if B[k] < n else np.float32(0.5)
        mat[r, 0] = mat[r, 1] = np.float32((fa + fb) * np.float32(0.5))
    return A[keep], B[keep], start, count, np.ascontiguousarray(packed, np.float32), mat


def run_tgs(which, scene, A, B, start, count, contacts, mat, dt=1.0 / 60.0, nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0),
            bounce=-2.0, friction_offset=0.04, correlation=0.025):
    """One TGS solve (construct, batch, prep, solve, integrate): returns velocities (n,6),
    poses (n,7), headers (start, stride) and the constraint order."""
    n = len(scene["types"])
    m = len(scene["static_poses"])
    nc = len(A)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nc, 1) * 2, np.uint32)
    hst = np.zeros(max(nc, 1) * 2, np.uint32)
    order = np.zeros(max(nc, 1), np.uint32)
    g = np.array(gravity, np.float32)
    L = oracle() if which == "orc" else reference()
    fn = L.orc_tgs_solve if which == "orc" else L.pxref_tgs_solve
    fn.restype = ctypes.c_uint32
    nh = fn(_p(scene["rigid"]), ctypes.c_uint32(n), _p(np.ascontiguousarray(scene["static_poses"], np.float32)), ctypes.c_uint32(m),
            _p(A), _p(B), ctypes.c_uint32(nc), _p(start), _p(count), _p(contacts), _p(mat), _p(g), ctypes.c_float(dt),
            ctypes.c_uint32(nb_pos), ctypes.c_uint32(nb_vel), ctypes.c_float(bounce), ctypes.c_float(friction_offset),
            ctypes.c_float(correlation), _p(vel), _p(pose), _p(hs), _p(hst), _p(order), None, None)
    return vel, pose, hs[:nh].copy(), hst[:nh].copy(), order[:nc].copy()


def run_pgs(which, scene, A, B, start, count, contacts, mat, dt=1.0 / 60.0, nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0),
            bounce=-2.0, friction_offset=0.04, correlation=0.025, batch=True):
    """One PGS solve (PxConstructSolverBodies, PxBatchConstraints or one header per
    constraint, PxCreateContactConstraints, PxSolveConstraints,
    PxIntegrateSolverBodies): returns velocities (n,6), poses (n,7), headers
    (start, stride, type), the constraint order and the written-back normal
    impulse per contact."""
    n = len(scene["types"])
    m = len(scene["static_poses"])
    nc = len(A)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nc, 1) * 2, np.uint32)
    hst = np.zeros(max(nc, 1) * 2, np.uint32)
    hty = np.zeros(max(nc, 1) * 2, np.uint32)
    order = np.zeros(max(nc, 1), np.uint32)
    forces = np.zeros(max(len(contacts), 1), np.float32)
    g = np.array(gravity, np.float32)
    L = oracle() if which == "orc" else reference()
    fn = L.orc_pgs_solve if which == "orc" else L.pxref_pgs_solve
    fn.restype = ctypes.c_uint32
    nh = fn(_p(scene["rigid"]), ctypes.c_uint32(n), _p(np.ascontiguousarray(scene["static_poses"], np.float32)), ctypes.c_uint32(m),
            _p(A), _p(B), ctypes.c_uint32(nc), _p(start), _p(count), _p(contacts), _p(mat), _p(g), ctypes.c_float(dt),
            ctypes.c_uint32(nb_pos), ctypes.c_uint32(nb_vel), ctypes.c_float(bounce), ctypes.c_float(friction_offset),
            ctypes.c_float(correlation), ctypes.c_int(1 if batch else 0), _p(vel), _p(pose), _p(hs), _p(hst), _p(hty), _p(order), _p(forces))
    return dict(vel=vel, pose=pose, header_start=hs[:nh].copy(), header_stride=hst[:nh].copy(), header_type=hty[:nh].copy(),
                order=order[:nc].copy(), forces=forces[:len(contacts)].copy())


def run_scene_step(which, scenes, params, steps=1):
    """Steps every scene `steps` times through the oracle ("orc") or the reference
    ("pxref"); returns the updated PxRigidBodyData array."""
    import sys
    sys.path.insert(0, ROOT)
    from physx_gb300.world import param_vector
    pv, it = param_vector(params)
    rb = np.ascontiguousarray(scenes["rigid"]).copy()
    L = oracle() if which == "orc" else reference()
    fn = L.orc_scene_step if which == "orc" else L.pxref_scene_step
    keep = [np.ascontiguousarray(scenes[k], d) for k, d in (("body_count", np.uint32), ("static_count", np.uint32), ("types", np.int32),
                                                              ("geoms", np.float32), ("friction", np.float32), ("static_poses", np.float32),
                                                              ("static_types", np.int32), ("static_geoms", np.float32))]
    for _ in range(steps):
        fn(ctypes.c_uint32(len(keep[0])), _p(keep[0]), _p(keep[1]), _p(rb), _p(keep[2]), _p(keep[3]), _p(keep[4]), _p(keep[5]),
           _p(keep[6]), _p(keep[7]), _p(pv), _p(it))
    return rb


class CachedContacts:
    """PxGenerateContacts over the same pairs frame after frame with persistent caches
    (PCM manifolds carried between calls): the oracle keeps 288-byte manifold records,
    the reference build its own PxCache array."""

    def __init__(self, which, n):
        self.which, self.n = which, n
        if which == "orc":
            self.L = oracle()
            self.state = np.zeros(n * 288, np.uint8)
        else:
            self.L = reference()
            self.L.pxref_np_create.restype = ctypes.c_void_p
            self.ctx = ctypes.c_void_p(self.L.pxref_np_create(ctypes.c_uint32(n)))

    def run(self, pairs, contact_distance=0.04, mesh_margin=0.01, tolerance_length=1.0, max_per_pair=8):
        n = self.n
        out = np.zeros((n, max_per_pair, 8), np.float32)
        cnt = np.zeros(n, np.uint32)
        args = [_p(np.ascontiguousarray(pairs[k])) for k in ("type0", "geom0", "type1", "geom1", "pose0", "pose1")]
        if self.which == "orc":
            rc = self.L.orc_np_run_cached(*args, ctypes.c_uint32(n), ctypes.c_float(contact_distance), ctypes.c_float(mesh_margin),
                                          ctypes.c_float(tolerance_length), _p(out), ctypes.c_uint32(max_per_pair), _p(cnt),
                                          _p(self.state))
        else:
            rc = self.L.pxref_np_run(self.ctx, *args, ctypes.c_uint32(n), ctypes.c_float(contact_distance), ctypes.c_float(mesh_margin),
                                     ctypes.c_float(tolerance_length), 0, _p(out), ctypes.c_uint32(max_per_pair), _p(cnt))
        assert rc == 0, "contact buffer overflow"
        return cnt, out

    def release(self):
        if self.which != "orc" and self.ctx:
            self.L.pxref_np_release(self.ctx)
            self.ctx = None


class PersistentScenes:
    """Scene frames with persistent pair state (contact caches and friction data
    carried between frames, the snippet's WITH_PERSISTENCY mode) through the oracle
    ("orc") or the reference ("pxref")."""

    def __init__(self, which, scenes, params):
        import sys
        sys.path.insert(0, ROOT)
        from physx_gb300.world import param_vector
        self.which = which
        self.pv, self.it = param_vector(params)
        self.L = oracle() if which == "orc" else reference()
        create = self.L.orc_persistent_create if which == "orc" else self.L.pxref_persistent_create
        create.restype = ctypes.c_void_p
        self.h = ctypes.c_void_p(create())
        self.fn = self.L.orc_scene_step_persistent if which == "orc" else self.L.pxref_scene_step_persistent
        self.keep = [np.ascontiguousarray(scenes[k], d) for k, d in (("body_count", np.uint32), ("static_count", np.uint32),
                                                                       ("types", np.int32), ("geoms", np.float32), ("friction", np.float32),
                                                                       ("static_poses", np.float32), ("static_types", np.int32),
                                                                       ("static_geoms", np.float32))]
        self.rb = np.ascontiguousarray(scenes["rigid"]).copy()

    def step(self, steps=1):
        k = self.keep
        for _ in range(steps):
            self.fn(self.h, ctypes.c_uint32(len(k[0])), _p(k[0]), _p(k[1]), _p(self.rb), _p(k[2]), _p(k[3]), _p(k[4]), _p(k[5]), _p(k[6]),
                    _p(k[7]), _p(self.pv), _p(self.it))
        return self.rb

    def release(self):
        if self.h:
            (self.L.orc_persistent_release if self.which == "orc" else self.L.pxref_persistent_release)(self.h)
            self.h = None


def run_joints(which, frame, dt=1.0 / 60.0, nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0), batch=True):
    """One TGS frame of joints (construct, batch, PxCreateJointConstraintsTGS,
    solve, integrate) through the oracle ("orc") or the reference ("pxref").
    frame: dict of nb_dyn, static_poses, joint_a, joint_b, rigid (PxRigidBodyData),
    rows (Px1DConstraint), row_start, row_count, params (see joint_scenes.joint_frame).
    Returns velocities (n,6), poses (n,7), headers (start, stride, type), the
    joint order, per-joint impulses (J,6) and broken flags.  batch=False: one
    header of stride 1 per joint in input order."""
    A = np.ascontiguousarray(frame["joint_a"], np.uint32)
    B = np.ascontiguousarray(frame["joint_b"], np.uint32)
    n = int(frame["nb_dyn"])
    m = len(frame["static_poses"])
    nj = len(A)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nj, 1), np.uint32)
    hst = np.zeros(max(nj, 1), np.uint32)
    ht = np.zeros(max(nj, 1), np.uint32)
    order = np.zeros(max(nj, 1), np.uint32)
    force = np.zeros((max(nj, 1), 6), np.float32)
    broken = np.zeros(max(nj, 1), np.uint32)
    g = np.array(gravity, np.float32)
    L = oracle() if which == "orc" else reference()
    fn = L.orc_joint_frame if which == "orc" else L.pxref_joint_frame
    fn.restype = ctypes.c_uint32
    rb = np.ascontiguousarray(frame["rigid"])
    nh = fn(_p(rb), ctypes.c_uint32(n), _p(np.ascontiguousarray(frame["static_poses"], np.float32)), ctypes.c_uint32(m), _p(A), _p(B),
            ctypes.c_uint32(nj), _p(np.ascontiguousarray(frame["row_start"], np.uint32)), _p(np.ascontiguousarray(frame["row_count"], np.uint32)),
            _p(np.ascontiguousarray(frame["rows"])), _p(np.ascontiguousarray(frame["params"], np.float32)), _p(g), ctypes.c_float(dt),
            ctypes.c_uint32(nb_pos), ctypes.c_uint32(nb_vel), ctypes.c_uint32(1 if batch else 0), _p(vel), _p(pose), _p(hs), _p(hst), _p(ht),
            _p(order), _p(force), _p(broken))
    return dict(vel=vel, pose=pose, header_start=hs[:nh].copy(), header_stride=hst[:nh].copy(), header_type=ht[:nh].copy(),
                order=order[:nj].copy(), force=force[:nj].copy(), broken=broken[:nj].copy())


def advance_rigid(rigid, vel, pose):
    """PxRigidBodyData for the next frame from a frame's velocities and poses."""
    out = rigid.copy()
    out["linVel"] = vel[:, :3]
    out["angVel"] = vel[:, 3:]
    out["q"] = pose[:, :4]
    out["p"] = pose[:, 4:]
    return out
