"""Long-horizon check on physical statistics (chaotic divergence makes per-body
comparison meaningless after a few hundred steps): the 210-box pyramid of the
reference's immediate-mode snippet, 300 steps at dt = 1/60, against the
reference's own trace (tests/golden/pyramid_stats.npz, made by
tests/golden/make_golden.py).  Stated bounds:

* peak kinetic energy within 10 %, time-averaged kinetic energy within 15 %;
* settled stack height (highest box centre at the end) within 0.05 m;
* penetration into the ground: the lowest box centre never more than 5 mm below
  the reference's lowest;
* mean horizontal drift of the boxes within 25 %.
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pyramid_stats.npz")
GOLDEN_PERSISTENT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pyramid_stats_persistent.npz")
STEPS = 300


def check_stats(ref, ke, top, low, drift):
    assert abs(ke.max() - ref["ke"].max()) <= 0.10 * ref["ke"].max(), (ke.max(), ref["ke"].max())
    assert abs(ke.mean() - ref["ke"].mean()) <= 0.15 * ref["ke"].mean(), (ke.mean(), ref["ke"].mean())
    assert abs(top[-1] - ref["top"][-1]) <= 0.05, (top[-1], ref["top"][-1])
    assert low.min() >= ref["low"].min() - 0.005, (low.min(), ref["low"].min())
    assert abs(drift - float(ref["drift"])) <= 0.25 * float(ref["drift"]), (drift, float(ref["drift"]))


def test_oracle_pyramid_statistics_match_reference():
    from oracle_libs import run_scene_step
    from physx_gb300.workloads import kinetic_energy, pyramid_scene
    from physx_gb300.world import DEFAULT_PARAMS
    ref = np.load(GOLDEN)
    sc = pyramid_scene()
    rb = sc["rigid"].copy()
    ke, top, low = [], [], []
    for _ in range(STEPS):
        rb = run_scene_step("orc", dict(sc, rigid=rb), DEFAULT_PARAMS, steps=1)
        ke.append(kinetic_energy(rb))
        top.append(rb["p"][:, 1].max())
        low.append(rb["p"][:, 1].min())
    check_stats(ref, np.array(ke), np.array(top), np.array(low), float(np.abs(rb["p"][:, 0] - sc["rigid"]["p"][:, 0]).mean()))
    # the oracle follows the reference's arithmetic exactly: its 300-step trace is the reference's
    assert np.array_equal(np.array(ke), ref["ke"]) and np.array_equal(np.array(top), ref["top"])
    assert np.array_equal(np.array(low), ref["low"])


def test_oracle_pyramid_persistent_trace_equals_reference():
    """The snippet's default mode: contact caches and friction data persist between
    frames.  The oracle's 300-step trace is the reference's, bit for bit."""
    from oracle_libs import PersistentScenes
    from physx_gb300.workloads import kinetic_energy, pyramid_scene
    from physx_gb300.world import DEFAULT_PARAMS
    ref = np.load(GOLDEN_PERSISTENT)
    sc = pyramid_scene()
    ps = PersistentScenes("orc", sc, DEFAULT_PARAMS)
    ke, top, low = [], [], []
    for _ in range(STEPS):
        rb = ps.step()
        ke.append(kinetic_energy(rb))
        top.append(rb["p"][:, 1].max())
        low.append(rb["p"][:, 1].min())
    ps.release()
    assert np.array_equal(np.array(ke), ref["ke"]) and np.array_equal(np.array(top), ref["top"])
    assert np.array_equal(np.array(low), ref["low"])


@pytest.mark.gpu
@pytest.mark.parametrize("persistent", [True, False])
def test_world_pyramid_statistics_match_reference(cuda_device, persistent):
    """The world in the snippet's persistent mode against the reference's persistent
    trace, and with fresh caches against the fresh trace."""
    from physx_gb300.workloads import kinetic_energy, pyramid_scene
    from physx_gb300.world import World
    ref = np.load(GOLDEN_PERSISTENT if persistent else GOLDEN)
    sc = pyramid_scene()
    w = World(sc, persistent=persistent)
    ke, top, low = [], [], []
    for _ in range(STEPS):
        w.step(1)
        rb = w.get_bodies()
        ke.append(kinetic_energy(rb))
        top.append(rb["p"][:, 1].max())
        low.append(rb["p"][:, 1].min())
    assert not w.status().any()
    w.release()
    check_stats(ref, np.array(ke), np.array(top), np.array(low), float(np.abs(rb["p"][:, 0] - sc["rigid"]["p"][:, 0]).mean()))
