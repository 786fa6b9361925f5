"""GB300 broadphase parity: created/lost pair sets bit-exact with the reference
ABP (golden fixtures) and with the CPU oracle on larger seeded inputs."""
import numpy as np
import pytest

from oracle_libs import CpuBroadPhase
from scenarios import bp_frames, sorted_pairs
from test_oracle_golden import BP_FIXTURES, load_bp_fixture

pytestmark = pytest.mark.gpu


def _gpu_bp():
    from physx_gb300.broadphase import BroadPhase
    return BroadPhase()


def _run(bp, fr):
    bp.update(fr["created"], fr["updated"], fr["removed"], fr["bounds"], fr["groups"], fr["distances"], fr["capacity"])
    return bp.fetch_results()


@pytest.mark.parametrize("path", BP_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in BP_FIXTURES])
@pytest.mark.parametrize("tiled", [True, False], ids=["tiled", "per-box"])
def test_bp_matches_reference_golden(cuda_device, path, tiled):
    bp = _gpu_bp()
    bp.set_sweep(tiled)
    for f, fr in enumerate(load_bp_fixture(path)):
        created, lost = _run(bp, fr)
        # bit-exact sets; the GB300 lists also come out already sorted
        assert np.array_equal(created, sorted_pairs(fr["ref_created"])), "frame %d created" % f
        assert np.array_equal(lost, sorted_pairs(fr["ref_lost"])), "frame %d lost" % f
    bp.release()


@pytest.mark.parametrize("tiled", [True, False], ids=["tiled", "per-box"])
@pytest.mark.parametrize("seed,n,frames,extent,move", [(31, 20000, 4, 60.0, 0.1), (32, 100000, 3, 300.0, 0.1),
                                                         (33, 5000, 6, 8.0, 0.5),
                                                         # X ranges over ~1600 sorted positions (several shared-memory
                                                         # tiles), with updated boxes sparse and then nearly all
                                                         (34, 30000, 3, 20.0, 0.01), (35, 30000, 3, 20.0, 0.9)])
def test_bp_matches_oracle(cuda_device, seed, n, frames, extent, move, tiled):
    bp, orc = _gpu_bp(), CpuBroadPhase("orc")
    bp.set_sweep(tiled)
    for f, fr in enumerate(bp_frames(seed, n, frames, extent=extent, move_frac=move)):
        gc, gl = _run(bp, fr)
        oc, ol = orc.update(fr)
        assert np.array_equal(gc, sorted_pairs(oc)), "frame %d created" % f
        assert np.array_equal(gl, sorted_pairs(ol)), "frame %d lost" % f
    bp.release()
    orc.release()


def test_bp_broadphase_stress_size(cuda_device):
    """1M boxes in a 1000 m cube, half-extents log-normal(ln 0.5, 0.5), 10% moved by
    N(0, 0.2) per frame, all dynamic, distance 0 (the broadphase-stress workload):
    20 consecutive update frames after the creating one, each frame's created and
    lost sets equal to the oracle ABP's."""
    n = 1_000_000
    bp, orc = _gpu_bp(), CpuBroadPhase("orc")
    for f, fr in enumerate(bp_frames(3, n, 21, extent=1000.0, move_frac=0.1, edge_cases=False, removals=False, distances=False)):
        fr["groups"] = ((np.arange(n, dtype=np.uint32) + 1) << 3) | 2
        gc, gl = _run(bp, fr)
        oc, ol = orc.update(fr)
        assert np.array_equal(gc, sorted_pairs(oc)), "frame %d created" % f
        assert np.array_equal(gl, sorted_pairs(ol)), "frame %d lost" % f
        st = bp.stats()
        assert st["live"] == n
    bp.release()
    orc.release()


def test_bp_deterministic_and_edge_cases(cuda_device):
    from physx_gb300 import GbpxError
    frames = list(bp_frames(41, 3000, 4, extent=20.0))
    a, b = _gpu_bp(), _gpu_bp()
    for fr in frames:
        ra, rb = _run(a, fr), _run(b, fr)
        assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])
    # empty update: nothing created or lost, state kept
    empty = dict(frames[-1])
    empty.update(created=np.zeros(0, np.uint32), updated=np.zeros(0, np.uint32), removed=np.zeros(0, np.uint32))
    c, l = _run(a, empty)
    assert len(c) == 0 and len(l) == 0
    # fetch without update is a call-sequence error, as is update twice
    with pytest.raises(GbpxError):
        a.fetch_results()
    a.update(empty["created"], empty["updated"], empty["removed"], empty["bounds"], empty["groups"], empty["distances"],
             empty["capacity"])
    with pytest.raises(GbpxError):
        a.update(empty["created"], empty["updated"], empty["removed"], empty["bounds"], empty["groups"], empty["distances"],
                 empty["capacity"])
    a.fetch_results()
    # removing everything loses nothing (pairs with removed objects are dropped silently)
    live = set()
    for fr in frames:
        live |= set(fr["created"].tolist())
        live -= set(fr["removed"].tolist())
    gone = dict(frames[-1])
    gone.update(created=np.zeros(0, np.uint32), updated=np.zeros(0, np.uint32),
                removed=np.array(sorted(live), np.uint32))
    orc = CpuBroadPhase("orc")
    for fr in frames:
        orc.update(fr)
    oc, ol = orc.update(gone)
    c, l = _run(a, gone)
    assert np.array_equal(c, sorted_pairs(oc)) and np.array_equal(l, sorted_pairs(ol))
    # out-of-range handle is rejected without touching the device
    bad = dict(frames[-1])
    bad.update(created=np.array([bad["capacity"] + 5], np.uint32), updated=np.zeros(0, np.uint32), removed=np.zeros(0, np.uint32))
    with pytest.raises(GbpxError):
        _run(b, bad)
    a.release()
    b.release()
