"""GB300 PGS frames (gbpx_pgs_solve: PxConstructSolverBodies, PxBatchConstraints,
PxCreateContactConstraints with the per-pair and the 4-wide block paths,
PxSolveConstraints, PxIntegrateSolverBodies) against the reference's own frames
(tests/golden/pgs_*.npz) and against the CPU oracle on larger seeded piles:
headers, their types and the constraint order exactly; body velocities within
1e-5 relative (per body, against max(|v|, 1e-2)), poses within 1e-6 and the
written-back normal impulses within 1e-5 relative (per contact, against
max(|impulse|, 1e-2)).  The integration evaluates sine and cosine with the
device's functions, so poses and velocities differ from the CPU's by rounding
only."""
import numpy as np
import pytest

from oracle_libs import run_pgs, scene_contacts, scene_pairs
from scenarios import random_scene
from test_oracle_golden import PGS_FIXTURES, pgs_fixture_args, velocity_error

pytestmark = pytest.mark.gpu


def force_error(ref, got):
    return float((np.abs(ref - got) / np.maximum(np.abs(ref), 1e-2)).max()) if len(ref) else 0.0


def assert_pgs_close(ref, got, what):
    for k in ("header_start", "header_stride", "header_type", "order"):
        assert np.array_equal(got[k], ref[k]), "%s: %s" % (what, k)
    assert velocity_error(ref["vel"], got["vel"]) <= 1e-5, what
    assert np.abs(ref["pose"] - got["pose"]).max() <= 1e-6, what
    assert force_error(ref["forces"], got["forces"]) <= 1e-5, what


def gpu_pgs(sc, a, b, s, c, ct, mat, **kw):
    from physx_gb300.solver import pgs_step
    return pgs_step(sc["rigid"], sc["static_poses"], a, b, s, c, ct, mat, **kw)


@pytest.mark.parametrize("batch", [True, False], ids=["batched", "one header per constraint"])
@pytest.mark.parametrize("path", PGS_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in PGS_FIXTURES])
def test_pgs_matches_reference_golden(cuda_device, path, batch):
    sc, z, args = pgs_fixture_args(path)
    tag = "batched" if batch else "single"
    ref = {k: z["ref_%s_%s" % (tag, k)] for k in ("vel", "pose", "header_start", "header_stride", "header_type", "order", "forces")}
    assert_pgs_close(ref, gpu_pgs(sc, *args, batch=batch), path)


@pytest.mark.parametrize("seed,n,restitution,iters", [(71, 400, 0.0, (4, 1)), (72, 1500, 0.3, (4, 1)), (73, 600, 0.0, (8, 3)),
                                                      (74, 200, 0.5, (1, 1))])
def test_pgs_matches_oracle(cuda_device, seed, n, restitution, iters):
    sc = random_scene(seed, n)
    A, B = scene_pairs(sc)
    a, b, s, c, ct, mat = scene_contacts("orc", sc, A, B)
    mat[:, 2] = restitution
    for batch in (True, False):
        ref = run_pgs("orc", sc, a, b, s, c, ct, mat, batch=batch, nb_pos=iters[0], nb_vel=iters[1])
        got = gpu_pgs(sc, a, b, s, c, ct, mat, batch=batch, nb_pos=iters[0], nb_vel=iters[1])
        assert_pgs_close(ref, got, "seed %d batch %s" % (seed, batch))
        if batch:
            assert {6, 7} & set(got["header_type"].tolist())   # block headers are in the batch


def test_pgs_edge_cases(cuda_device):
    from physx_gb300 import GbpxError
    sc = random_scene(75, 30)
    A, B = scene_pairs(sc)
    a, b, s, c, ct, mat = scene_contacts("orc", sc, A, B)
    # no constraints: free fall only
    empty = np.zeros(0, np.uint32)
    got = gpu_pgs(sc, empty, empty, empty, empty, np.zeros((0, 8), np.float32), np.zeros((0, 3), np.float32))
    ref = run_pgs("orc", sc, empty, empty, empty, empty, np.zeros((1, 8), np.float32), np.zeros((1, 3), np.float32))
    assert velocity_error(ref["vel"], got["vel"]) <= 1e-5 and len(got["header_start"]) == 0
    # a constraint with more than 4 contacts, or without one, is refused
    bad = c.copy()
    bad[0] = 5
    with pytest.raises(GbpxError):
        gpu_pgs(sc, a, b, s, bad, ct, mat)
    bad[0] = 0
    with pytest.raises(GbpxError):
        gpu_pgs(sc, a, b, s, bad, ct, mat)
