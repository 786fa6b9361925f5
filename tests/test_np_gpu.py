"""GB300 narrowphase parity: against the reference's PxGenerateContacts
(golden fixture) and the CPU oracle on larger seeded batches."""
import numpy as np
import pytest

from contact_compare import assert_report, compare, unpack
from oracle_libs import run_contacts
from scenarios import np_pairs
from test_oracle_golden import NP_FIXTURES, load_np_fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", NP_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in NP_FIXTURES])
def test_contacts_match_reference_golden(cuda_device, path):
    from physx_gb300.contacts import generate_contacts
    pairs, rc, rpacked, cd, tl = load_np_fixture(path)
    gc, go = generate_contacts(pairs, contact_distance=cd, tolerance_length=tl, max_per_pair=4)
    rep = compare(pairs, rc, unpack(rc, rpacked), gc, [go[i, :gc[i]] for i in range(len(gc))])
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
