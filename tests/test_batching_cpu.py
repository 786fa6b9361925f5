"""PxBatchConstraintsTGS on the host (gbpx_batch_constraints_tgs, batching.h)
against the oracle's restatement on random constraint sets: headers and order
equal, including multi-round overflow (bodies in more than 32 constraints) and
static constraints.  Host code only: runs without a GPU."""
import ctypes

import numpy as np
import pytest


def _oracle_batch(a, b, nd, ns):
    from oracle_libs import oracle
    L = oracle()
    n = len(a)
    hs = np.zeros(max(n, 1), np.uint32)
    hst = np.zeros(max(n, 1), np.uint32)
    order = np.zeros(max(n, 1), np.uint32)
    P = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    L.orc_batch_constraints_tgs.restype = ctypes.c_uint32
    nh = L.orc_batch_constraints_tgs(P(a), P(b), ctypes.c_uint32(n), ctypes.c_uint32(nd), ctypes.c_uint32(ns), P(hs), P(hst), P(order))
    return hs[:nh], hst[:nh], order[:n]


@pytest.mark.parametrize("seed,nd,ns,n,hubs", [(1, 200, 1, 600, 0), (2, 5000, 3, 20000, 0), (3, 300, 2, 2500, 4), (4, 50, 1, 1200, 2)])
def test_host_batching_matches_oracle(gbpx_built, seed, nd, ns, n, hubs):
    from physx_gb300.solver import batch_constraints
    rng = np.random.default_rng(seed)
    a = rng.integers(0, nd, n).astype(np.uint32)
    b = rng.integers(0, nd + ns, n).astype(np.uint32)
    if hubs:
        # a few bodies in many constraints: several rounds of 32 partitions
        a[: n // 3] = rng.integers(0, hubs, n // 3)
    keep = a != b
    a, b = np.minimum(a[keep], b[keep]), np.maximum(a[keep], b[keep])
    hs, hst, order = batch_constraints(a, b, nd, ns)
    ohs, ohst, oorder = _oracle_batch(a, b, nd, ns)
    assert np.array_equal(hs, ohs) and np.array_equal(hst, ohst) and np.array_equal(order, oorder)
    if hubs:
        assert len(hs) > 0
