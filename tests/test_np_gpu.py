"""GB300 narrowphase parity: against the reference's PxGenerateContacts
(golden fixture) and the CPU oracle on larger seeded batches."""
import numpy as np
import pytest

from contact_compare import assert_report, compare, unpack
from oracle_libs import run_contacts
from scenarios import np_pairs
from test_oracle_golden import NP_FIXTURES, load_np_fixture
from physx_gb300.workloads import convex_core_pairs, convex_core_type

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", NP_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in NP_FIXTURES])
def test_contacts_match_reference_golden(cuda_device, path):
    from physx_gb300.contacts import generate_contacts
    pairs, rc, rpacked, cd, tl = load_np_fixture(path)
    gc, go = generate_contacts(pairs, contact_distance=cd, tolerance_length=tl, max_per_pair=4)
    rep = compare(pairs, rc, unpack(rc, rpacked), gc, [go[i, :gc[i]] for i in range(len(gc))])
    print({k: r["maxdiff"] for k, r in rep.items()})
    assert_report(rep)


@pytest.mark.parametrize("seed,n", [(101, 20000), (102, 2000)])
def test_contacts_match_oracle(cuda_device, seed, n):
    from physx_gb300.contacts import generate_contacts
    pairs = np_pairs(seed, n)
    gc, go = generate_contacts(pairs, max_per_pair=4)
    oc, oo = run_contacts("orc", pairs, max_per_pair=4)
    assert np.array_equal(gc, oc)
    for i in np.flatnonzero(oc):
        assert np.abs(go[i, :oc[i], :7] - oo[i, :oc[i], :7]).max() <= 1e-6, i


def _exact(pairs, gc, go, oc, oo):
    """Same counts; every value bit-identical, except on the pairs whose contact
    face is a cylinder's or cone's cap: rotatePoints turns those faces by an
    angle from acos and a quaternion from sin/cos, which the device evaluates in
    double and rounds while the oracle calls the host C library (as the
    reference does), so they may differ in the last bits; those pairs are held
    to the contact tolerance."""
    from contact_compare import CONTACT_TOL
    assert np.array_equal(gc, oc)
    cores = np.where((pairs["type0"] & 0xff) == 4, pairs["type0"] >> 8, -1), np.where((pairs["type1"] & 0xff) == 4, pairs["type1"] >> 8, -1)
    trig = np.isin(cores[0], (4, 5)) | np.isin(cores[1], (4, 5))
    for i in np.flatnonzero(oc):
        if trig[i]:
            assert np.abs(go[i, :oc[i], :7] - oo[i, :oc[i], :7]).max() <= CONTACT_TOL, i
        else:
            assert np.array_equal(go[i, :oc[i], :7], oo[i, :oc[i], :7]), i


@pytest.mark.parametrize("seed,n", [(103, 20000), (104, 3000)])
def test_convex_core_contacts_match_oracle(cuda_device, seed, n):
    """Convex cores of every type against every shape type, both argument orders:
    the same counts and bit-identical normals, separations and points."""
    from physx_gb300.contacts import generate_contacts
    pairs = convex_core_pairs(seed, n, aligned_frac=0.6)
    gc, go = generate_contacts(pairs, max_per_pair=4)
    oc, oo = run_contacts("orc", pairs, max_per_pair=4)
    assert (oc > 1).sum() > n // 20   # face contacts (2-4 points) are in the mix
    _exact(pairs, gc, go, oc, oo)


def test_mixed_primitive_and_convex_core_batch(cuda_device):
    """One batch with primitive and convex-core pairs interleaved: each pair's
    contacts come from its own generator (the buckets split the batch)."""
    from physx_gb300.contacts import generate_contacts
    a, b = np_pairs(105, 4000), convex_core_pairs(106, 4000)
    order = np.random.default_rng(107).permutation(8000)
    pairs = {k: np.concatenate([a[k], b[k]])[order] for k in a}
    gc, go = generate_contacts(pairs, max_per_pair=4)
    oc, oo = run_contacts("orc", pairs, max_per_pair=4)
    _exact(pairs, gc, go, oc, oo)


def test_convex_core_edge_cases(cuda_device):
    from physx_gb300 import GbpxError
    from physx_gb300.contacts import generate_contacts
    ident = np.array([0, 0, 0, 1, 0, 0, 0], np.float32)
    up = np.array([0, 0, 0, 1, 0, 0.95, 0], np.float32)
    s = np.float32(np.sqrt(0.5))
    plane = np.array([0, 0, s, s, 0, 0, 0], np.float32)
    cases = [
        # coincident point cores (spheres): EPA on a degenerate polytope
        (convex_core_type(0), [0, 0, 0, 0.5], ident, convex_core_type(0), [0, 0, 0, 0.5], ident),
        # a zero-size box core with no margin against a plane, touching
        (convex_core_type(2), [0, 0, 0, 0], ident, 1, [0, 0, 0, 0], plane),
        # a flat box (a rectangle) resting on a box core: face contact
        (convex_core_type(2), [1, 0, 1, 0.05], up, convex_core_type(2), [2, 1.8, 2, 0], ident),
        # a cylinder on its cap, a cone on its base against a plane
        (1, [0, 0, 0, 0], plane, convex_core_type(4), [1.0, 0.5, 0, 0], np.array([0, 0, s, s, 0, 0.49, 0], np.float32)),
        (1, [0, 0, 0, 0], plane, convex_core_type(5), [1.0, 0.5, 0, 0], np.array([0, 0, s, s, 0, 0.51, 0], np.float32)),
        # far apart: no contact
        (convex_core_type(3), [0.5, 0.2, 0.3, 0], ident, 3, [0.5, 0.5, 0.5, 0], np.array([0, 0, 0, 1, 9, 0, 0], np.float32)),
    ]
    pairs = dict(type0=np.array([c[0] for c in cases], np.int32), geom0=np.array([c[1] for c in cases], np.float32),
                 type1=np.array([c[3] for c in cases], np.int32), geom1=np.array([c[4] for c in cases], np.float32),
                 pose0=np.stack([c[2] for c in cases]), pose1=np.stack([c[5] for c in cases]))
    gc, go = generate_contacts(pairs, max_per_pair=4)
    oc, oo = run_contacts("orc", pairs, max_per_pair=4)
    _exact(pairs, gc, go, oc, oo)
    assert gc[-1] == 0 and gc[2] >= 2 and gc[3] == 4
    # an unknown core type and a core type on a primitive are rejected
    for bad in (convex_core_type(6), 3 | (2 << 8)):
        b = dict(pairs)
        b["type0"] = pairs["type0"].copy()
        b["type0"][0] = bad
        with pytest.raises(GbpxError):
            generate_contacts(b)


def test_contacts_edge_cases(cuda_device):
    from physx_gb300 import GbpxError
    from physx_gb300.contacts import generate_contacts
    # empty batch
    empty = {k: np.zeros((0, w), np.float32) if w else np.zeros(0, np.int32)
             for k, w in (("type0", 0), ("geom0", 4), ("type1", 0), ("geom1", 4), ("pose0", 7), ("pose1", 7))}
    c, o = generate_contacts(empty)
    assert len(c) == 0
    # plane vs plane gives no contact; coincident spheres get the +x fallback normal
    pl = np.array([0, 0, 0, 1, 0, 0, 0], np.float32)
    pairs = dict(type0=np.array([1, 0], np.int32), geom0=np.array([[0, 0, 0, 0], [0.5, 0, 0, 0]], np.float32),
                 type1=np.array([1, 0], np.int32), geom1=np.array([[0, 0, 0, 0], [0.5, 0, 0, 0]], np.float32),
                 pose0=np.stack([pl, pl]), pose1=np.stack([pl, pl]))
    c, o = generate_contacts(pairs)
    oc, oo = run_contacts("orc", pairs)
    assert c[0] == 0 and c[1] == 1 and np.allclose(o[1, 0, :3], [1, 0, 0]) and np.allclose(o[1, 0, :7], oo[1, 0, :7])
    # invalid geometry type is rejected
    bad = dict(pairs)
    bad["type0"] = np.array([7, 0], np.int32)
    with pytest.raises(GbpxError):
        generate_contacts(bad)


def test_cached_contacts_match_reference_golden(cuda_device):
    """Persistent caches over 8 moving frames (pcm_cached.npz, the reference's own
    outputs): same counts every frame, every value within the contact tolerance."""
    from contact_compare import CONTACT_TOL
    from physx_gb300.contacts import CachedContacts
    from test_oracle_golden import GOLDEN, load_np_cached_fixture
    import os
    pairs, frames = load_np_cached_fixture(os.path.join(GOLDEN, "pcm_cached.npz"))
    n = len(pairs["type0"])
    gpu = CachedContacts(n)
    for f, fr in enumerate(frames):
        gc, go = gpu.run(dict(pairs, pose0=fr["pose0"], pose1=fr["pose1"]))
        assert np.array_equal(gc, fr["counts"]), "frame %d" % f
        ref = unpack(fr["counts"], fr["contacts"])
        for i in np.flatnonzero(gc):
            assert np.abs(go[i, :gc[i], :7] - ref[i][:, :7]).max() <= CONTACT_TOL, (f, i)


def test_cached_contacts_match_oracle(cuda_device):
    from oracle_libs import CachedContacts as OracleCached
    from physx_gb300.contacts import CachedContacts
    from scenarios import moving_pairs
    pairs, poses = moving_pairs(105, 6000, 12)
    gpu, orc = CachedContacts(6000), OracleCached("orc", 6000)
    for p0, p1 in poses:
        fr = dict(pairs, pose0=p0, pose1=p1)
        gc, go = gpu.run(fr)
        oc, oo = orc.run(fr, max_per_pair=4)
        assert np.array_equal(gc, oc)
        for i in np.flatnonzero(oc):
            assert np.abs(go[i, :oc[i], :7] - oo[i, :oc[i], :7]).max() <= 1e-6, i
