"""The CPU oracle (oracle/port) against the reference's own outputs.

Golden fixtures in tests/golden were produced by the reference built from its
sources (tests/golden/make_golden.py).  Where that build is present (the
development machine), extra seeded cases are also compared live."""
import glob
import os

import numpy as np
import pytest

from oracle_libs import CpuBroadPhase, reference
from scenarios import bp_frames, sorted_pairs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_bp_fixture(path):
    z = np.load(path)
    frames = []
    for f in range(int(z["frames"])):
        fr = {k: z["f%d_%s" % (f, k)] for k in ("created", "updated", "removed", "bounds", "groups", "distances")}
        fr["capacity"] = int(z["f%d_capacity" % f])
        fr["ref_created"] = z["f%d_ref_created" % f]
        fr["ref_lost"] = z["f%d_ref_lost" % f]
        frames.append(fr)
    return frames


BP_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "bp_*.npz")))


@pytest.mark.parametrize("path", BP_FIXTURES, ids=[os.path.basename(p) for p in BP_FIXTURES])
def test_oracle_bp_matches_reference_golden(path):
    bp = CpuBroadPhase("orc")
    for f, fr in enumerate(load_bp_fixture(path)):
        created, lost = bp.update(fr)
        assert np.array_equal(sorted_pairs(created), sorted_pairs(fr["ref_created"])), "frame %d created" % f
        assert np.array_equal(sorted_pairs(lost), sorted_pairs(fr["ref_lost"])), "frame %d lost" % f
    bp.release()


def test_bp_fixtures_present():
    assert len(BP_FIXTURES) >= 2


@pytest.mark.skipif(reference() is None, reason="reference build (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("seed,n,frames,extent", [(21, 3000, 5, 40.0), (22, 200, 10, 5.0)])
def test_oracle_bp_matches_reference_live(seed, n, frames, extent):
    ref, orc = CpuBroadPhase("pxref"), CpuBroadPhase("orc")
    for fr in bp_frames(seed, n, frames, extent=extent):
        rc, rl = ref.update(fr)
        oc, ol = orc.update(fr)
        assert np.array_equal(sorted_pairs(rc), sorted_pairs(oc))
        assert np.array_equal(sorted_pairs(rl), sorted_pairs(ol))


NP_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "np_*.npz")))


def load_np_fixture(path):
    z = np.load(path)
    pairs = {k: z[k] for k in ("type0", "geom0", "type1", "geom1", "pose0", "pose1")}
    return pairs, z["counts"], z["contacts"], float(z["contact_distance"]), float(z["tolerance_length"])


@pytest.mark.parametrize("path", NP_FIXTURES, ids=[os.path.basename(p) for p in NP_FIXTURES])
def test_oracle_contacts_match_reference_golden(path):
    from contact_compare import assert_report, compare, unpack
    from oracle_libs import run_contacts
    pairs, rc, rpacked, cd, tl = load_np_fixture(path)
    oc, oo = run_contacts("orc", pairs, contact_distance=cd, tolerance_length=tl, max_per_pair=8)
    rep = compare(pairs, rc, unpack(rc, rpacked), oc, [oo[i, :oc[i]] for i in range(len(oc))])
    assert_report(rep)
    # the analytic pairs are reproduced bit for bit
    for k in ("sphere-sphere", "sphere-plane", "sphere-capsule", "sphere-box", "plane-capsule", "plane-box", "capsule-capsule"):
        assert rep[k]["maxdiff"] == 0.0, (k, rep[k])
