"""Immediate-mode TGS and PGS mirror over the GB300 solver kernels.

Mirrors physx/include/PxImmediateMode.h:592-729: PxConstructSolverBodiesTGS,
PxBatchConstraintsTGS and one full TGS step (PxCreateContactConstraintsTGS +
PxSolveConstraintsTGS + PxIntegrateSolverBodiesTGS) from given contacts; one
PGS frame (PxConstructSolverBodies, PxBatchConstraints,
PxCreateContactConstraints, PxSolveConstraints, PxIntegrateSolverBodies); joint
frames.
Rigid bodies are PxRigidBodyData records (numpy structured array, 96 bytes).
"""
import ctypes

import numpy as np

from . import check, lib

_p = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def _setup():
    L = lib()
    if not getattr(L, "_tgs_ready", False):
        L.gbpx_batch_constraints_tgs.restype = ctypes.c_uint32
        L.gbpx_batch_constraints_tgs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                                 ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_construct_solver_bodies_tgs.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_float,
                                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.gbpx_tgs_solve.argtypes = ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 5 +
                                     [ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float] + [ctypes.c_void_p] * 6)
        L._tgs_ready = True
    return L


def batch_constraints(body_a, body_b, nb_dynamic, nb_static=0):
    """Returns (header_start, header_stride, order)."""
    L = _setup()
    a = np.ascontiguousarray(body_a, np.uint32)
    b = np.ascontiguousarray(body_b, np.uint32)
    n = len(a)
    hs = np.zeros(max(n, 1), np.uint32)
    hst = np.zeros(max(n, 1), np.uint32)
    order = np.zeros(max(n, 1), np.uint32)
    nh = L.gbpx_batch_constraints_tgs(_p(a), _p(b), n, nb_dynamic, nb_static, _p(hs), _p(hst), _p(order))
    return hs[:nh].copy(), hst[:nh].copy(), order[:n].copy()


def construct_solver_bodies(rigid, gravity, dt):
    """Returns raw (PxTGSSolverBodyVel, PxTGSSolverBodyTxInertia, PxTGSSolverBodyData) records as float32 views."""
    L = _setup()
    rigid = np.ascontiguousarray(rigid)
    n = len(rigid)
    vel = np.zeros((n, 16), np.float32)
    tx = np.zeros((n, 16), np.float32)
    data = np.zeros((n, 12), np.float32)
    g = np.asarray(gravity, np.float32)
    check(L.gbpx_construct_solver_bodies_tgs(_p(rigid), n, _p(g), dt, _p(vel), _p(tx), _p(data)), "PxConstructSolverBodiesTGS")
    return vel, tx, data


def tgs_step(rigid, static_poses, body_a, body_b, contact_start, contact_count, contacts, material, dt=1.0 / 60.0,
             nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0), bounce=-2.0, friction_offset=0.04, correlation=0.025):
    """Returns (velocities (n,6), poses (n,7), header_start, header_stride, order)."""
    L = _setup()
    rigid = np.ascontiguousarray(rigid)
    n = len(rigid)
    sp = np.ascontiguousarray(static_poses, np.float32)
    a = np.ascontiguousarray(body_a, np.uint32)
    b = np.ascontiguousarray(body_b, np.uint32)
    nc = len(a)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nc, 1) * 2, np.uint32)
    hst = np.zeros(max(nc, 1) * 2, np.uint32)
    order = np.zeros(max(nc, 1), np.uint32)
    nh = ctypes.c_uint32(0)
    g = np.asarray(gravity, np.float32)
    check(L.gbpx_tgs_solve(_p(rigid), n, _p(sp), len(sp), _p(a), _p(b), nc,
                           _p(np.ascontiguousarray(contact_start, np.uint32)), _p(np.ascontiguousarray(contact_count, np.uint32)),
                           _p(np.ascontiguousarray(contacts, np.float32)), _p(np.ascontiguousarray(material, np.float32)), _p(g),
                           dt, nb_pos, nb_vel, bounce, friction_offset, correlation, _p(vel), _p(pose), _p(hs), _p(hst),
                           _p(order), ctypes.byref(nh)), "TGS step")
    return vel, pose, hs[:nh.value].copy(), hst[:nh.value].copy(), order[:nc].copy()


def pgs_step(rigid, static_poses, body_a, body_b, contact_start, contact_count, contacts, material, dt=1.0 / 60.0,
             nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0), bounce=-2.0, friction_offset=0.04, correlation=0.025, batch=True):
    """One PGS frame (PxConstructSolverBodies, PxBatchConstraints or one header per
    constraint, PxCreateContactConstraints, PxSolveConstraints,
    PxIntegrateSolverBodies): returns dict(vel (n,6), pose (n,7), header_start,
    header_stride, header_type, order, forces (per contact))."""
    L = lib()
    if not getattr(L, "_pgs_ready", False):
        L.gbpx_pgs_solve.argtypes = ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 5 +
                                     [ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_int] + [ctypes.c_void_p] * 8)
        L._pgs_ready = True
    rigid = np.ascontiguousarray(rigid)
    n = len(rigid)
    sp = np.ascontiguousarray(static_poses, np.float32)
    a = np.ascontiguousarray(body_a, np.uint32)
    b = np.ascontiguousarray(body_b, np.uint32)
    ct = np.ascontiguousarray(contacts, np.float32)
    nc = len(a)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nc, 1), np.uint32)
    hst = np.zeros(max(nc, 1), np.uint32)
    hty = np.zeros(max(nc, 1), np.uint32)
    order = np.zeros(max(nc, 1), np.uint32)
    forces = np.zeros(max(len(ct), 1), np.float32)
    nh = ctypes.c_uint32(0)
    g = np.asarray(gravity, np.float32)
    check(L.gbpx_pgs_solve(_p(rigid), n, _p(sp), len(sp), _p(a), _p(b), nc,
                           _p(np.ascontiguousarray(contact_start, np.uint32)), _p(np.ascontiguousarray(contact_count, np.uint32)),
                           _p(ct), _p(np.ascontiguousarray(material, np.float32)), _p(g), dt, nb_pos, nb_vel, bounce, friction_offset,
                           correlation, 1 if batch else 0, _p(vel), _p(pose), _p(hs), _p(hst), _p(hty), _p(order), _p(forces),
                           ctypes.byref(nh)), "PGS step")
    k = nh.value
    return dict(vel=vel, pose=pose, header_start=hs[:k].copy(), header_stride=hst[:k].copy(), header_type=hty[:k].copy(),
                order=order[:nc].copy(), forces=forces[:len(ct)].copy())


def joint_frame(frame, dt=1.0 / 60.0, nb_pos=4, nb_vel=1, gravity=(0.0, -9.81, 0.0), batch=True):
    """One TGS frame of joints on the GB300 (gbpx_joint_frame: construct bodies,
    PxBatchConstraintsTGS over the joints, PxCreateJointConstraintsTGS, solve,
    write-back, PxIntegrateSolverBodiesTGS).  frame: dict of nb_dyn,
    static_poses, joint_a, joint_b, rigid (PxRigidBodyData), rows
    (Px1DConstraint records, 80 bytes), row_start, row_count, params (20 floats
    per joint).  Returns velocities (n,6), poses (n,7), headers (start,
    stride, type), the joint order, per-joint impulses (J,6) and broken flags."""
    L = _setup()
    A = np.ascontiguousarray(frame["joint_a"], np.uint32)
    B = np.ascontiguousarray(frame["joint_b"], np.uint32)
    n = int(frame["nb_dyn"])
    statics = np.ascontiguousarray(frame["static_poses"], np.float32)
    nj = len(A)
    vel = np.zeros((n, 6), np.float32)
    pose = np.zeros((n, 7), np.float32)
    hs = np.zeros(max(nj, 1), np.uint32)
    hst = np.zeros(max(nj, 1), np.uint32)
    ht = np.zeros(max(nj, 1), np.uint32)
    order = np.zeros(max(nj, 1), np.uint32)
    force = np.zeros((max(nj, 1), 6), np.float32)
    broken = np.zeros(max(nj, 1), np.uint32)
    nh = np.zeros(1, np.uint32)
    g = np.asarray(gravity, np.float32)
    keep = [np.ascontiguousarray(frame["rigid"]), np.ascontiguousarray(frame["row_start"], np.uint32),
            np.ascontiguousarray(frame["row_count"], np.uint32), np.ascontiguousarray(frame["rows"]),
            np.ascontiguousarray(frame["params"], np.float32)]
    L.gbpx_joint_frame.argtypes = ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_uint32] + [ctypes.c_void_p] * 5 +
                                   [ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32] + [ctypes.c_void_p] * 9)
    check(L.gbpx_joint_frame(_p(keep[0]), n, _p(statics), len(statics), _p(A), _p(B), nj, _p(keep[1]), _p(keep[2]), _p(keep[3]), _p(keep[4]),
                             _p(g), dt, nb_pos, nb_vel, 1 if batch else 0, _p(vel), _p(pose), _p(hs), _p(hst), _p(ht), _p(order), _p(force),
                             _p(broken), _p(nh)), "gbpx_joint_frame")
    k = int(nh[0])
    return dict(vel=vel, pose=pose, header_start=hs[:k].copy(), header_stride=hst[:k].copy(), header_type=ht[:k].copy(),
                order=order[:nj].copy(), force=force[:nj].copy(), broken=broken[:nj].copy())
