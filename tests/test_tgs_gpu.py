"""GB300 TGS parity: batching rule, solver bodies and one full solve against
the reference (golden fixtures) and the CPU oracle."""
import numpy as np
import pytest

from oracle_libs import run_tgs, scene_contacts, scene_pairs
from scenarios import random_scene
from test_oracle_golden import TGS_FIXTURES, TGS_POSE_TOL, TGS_VEL_REL_TOL, load_tgs_fixture, velocity_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", TGS_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in TGS_FIXTURES])
def test_tgs_matches_reference_golden(cuda_device, path):
    from physx_gb300.solver import batch_constraints, construct_solver_bodies, tgs_step
    rb, z = load_tgs_fixture(path)
    n = len(rb)
    hs, hst, order = batch_constraints(z["body_a"], z["body_b"], n, len(z["static_poses"]))
    assert np.array_equal(hs, z["ref_header_start"]) and np.array_equal(hst, z["ref_header_stride"])
    assert np.array_equal(order, z["ref_order"])
    bv, btx, bd = construct_solver_bodies(rb, (0.0, -9.81, 0.0), 1.0 / 60.0)
    # PxTGSSolverBodyVel: linear, angular (momentum space), deltas, maxAngVel; TxInertia: dq, p, sqrtInvInertia
    for cols in ([0, 1, 2], [4, 5, 6], [8, 9, 10, 11], [12, 13, 14]):
        assert np.abs(bv[:, cols] - z["ref_body_vel"][:, cols]).max() <= 1e-6 * max(1.0, np.abs(z["ref_body_vel"][:, cols]).max())
    assert np.abs(btx - z["ref_body_txi"]).max() <= 1e-6
    assert np.array_equal(bd[:, [3, 7]], z["ref_body_data"][:, [3, 7]])   # maxContactImpulse, penBiasClamp
    assert np.abs(bd[:, [0, 1, 2, 4, 5, 6, 8]] - z["ref_body_data"][:, [0, 1, 2, 4, 5, 6, 8]]).max() <= 1e-6
    vel, pose, hs2, hst2, order2 = tgs_step(rb, z["static_poses"], z["body_a"], z["body_b"], z["contact_start"], z["contact_count"],
                                            z["contacts"], z["material"])
    assert np.array_equal(order2, z["ref_order"])
    assert velocity_error(z["ref_velocity"], vel) <= TGS_VEL_REL_TOL
    assert np.abs(pose - z["ref_pose"]).max() <= TGS_POSE_TOL


@pytest.mark.parametrize("seed,n", [(51, 40), (52, 300)])
def test_tgs_matches_oracle(cuda_device, seed, n):
    from physx_gb300.solver import tgs_step
    sc = random_scene(seed, n)
    A, B = scene_pairs(sc)
    a, b, s, c, ct, mat = scene_contacts("orc", sc, A, B)
    ov, op, ohs, ohst, oo = run_tgs("orc", sc, a, b, s, c, ct, mat)
    gv, gp, ghs, ghst, go = tgs_step(sc["rigid"], sc["static_poses"], a, b, s, c, ct, mat)
    assert np.array_equal(go, oo) and np.array_equal(ghs, ohs) and np.array_equal(ghst, ohst)
    # same arithmetic; only sin/cos in the integrator come from different libraries
    assert velocity_error(ov, gv) <= 1e-5
    assert np.abs(gp - op).max() <= 1e-6


def test_batching_overflow_and_edge_cases(cuda_device):
    """More than 32 dynamic constraints on one body overflow into a second round of
    partitions; statics follow each body's last dynamic partition."""
    from oracle_libs import oracle
    import ctypes
    from physx_gb300.solver import batch_constraints
    rng = np.random.default_rng(61)
    nd, ns = 80, 3
    A = [0] * 45 + list(rng.integers(0, nd, 300))
    B = list(range(1, 46)) + list(rng.integers(0, nd + ns, 300))
    A, B = np.array(A, np.uint32), np.array(B, np.uint32)
    keep = (A != B) & ~((A >= nd) & (B >= nd))
    A, B = A[keep], B[keep]
    hs, hst, order = batch_constraints(A, B, nd, ns)
    L = oracle()
    n = len(A)
    ohs, ohst, oo = (np.zeros(2 * n, np.uint32) for _ in range(3))
    L.orc_batch_constraints_tgs.restype = ctypes.c_uint32
    P = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    nh = L.orc_batch_constraints_tgs(P(A), P(B), ctypes.c_uint32(n), ctypes.c_uint32(nd), ctypes.c_uint32(ns), P(ohs), P(ohst), P(oo))
    assert np.array_equal(hs, ohs[:nh]) and np.array_equal(hst, ohst[:nh]) and np.array_equal(order, oo[:n])
    assert sorted(order.tolist()) == list(range(n))
    # empty input
    hs, hst, order = batch_constraints(np.zeros(0, np.uint32), np.zeros(0, np.uint32), 4)
    assert len(hs) == 0 and len(order) == 0
