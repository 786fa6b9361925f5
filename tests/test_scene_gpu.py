"""One large scene on the GB300 (gbpx_scene_*): the reference snippet's frame
over one scene with every stage spread over the GPU, the ABP broadphase of
gbpx_bp, PxBatchConstraintsTGS on the host.  Checked against the batched world
(the same arithmetic: identical bytes), against the CPU oracle frame by frame
(persistent and fresh), at the full 100k-body size against one oracle frame, and
over the full 600-step run on physical statistics against the reference's trace."""
import os

import numpy as np
import pytest

from oracle_libs import PersistentScenes, run_scene_step
from test_oracle_golden import rigid_velocity, velocity_error

pytestmark = pytest.mark.gpu


def _pile(seed, n):
    from scenarios import random_scene
    # n bodies spread over the plane, most of them touching it or each other
    return random_scene(seed, n)


@pytest.mark.parametrize("persistent", [True, False])
def test_scene_equals_world(cuda_device, persistent):
    """The large-scene step and the batched world produce the same bytes for the
    same scene over 12 steps (same device functions, same batching order)."""
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world
    from physx_gb300.world import World
    sc = _pile(131, 400)
    s = Scene(sc, persistent=persistent)
    w = World(as_world(sc), persistent=persistent)
    for step in range(12):
        s.step(1)
        w.step(1)
        a, b = s.get_bodies(), w.get_bodies()
        assert a.tobytes() == b.tobytes(), step
    assert s.stats()["constraints"] > 100
    s.release()
    w.release()


def test_scene_persistent_steps_match_oracle(cuda_device):
    """Persistent frames against the oracle's persistent frames, step by step; the
    oracle's bodies are set to the device's after every step (pair state stays each
    side's own), so last-ulp sin/cos differences cannot grow chaotically."""
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world
    from physx_gb300.world import DEFAULT_PARAMS
    sc = _pile(132, 3000)
    s = Scene(sc)
    orc = PersistentScenes("orc", as_world(sc), DEFAULT_PARAMS)
    for step in range(8):
        s.step(1)
        out = s.get_bodies()
        ref = orc.step().copy()
        orc.rb[:] = out
        assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5, step
        assert np.abs(out["p"] - ref["p"]).max() <= 1e-6, step
    st = s.stats()
    assert st["constraints"] > 1000 and st["partitions"] > 4
    orc.release()
    s.release()


def test_scene_fresh_step_matches_oracle(cuda_device):
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world
    from physx_gb300.world import DEFAULT_PARAMS
    sc = _pile(133, 2000)
    s = Scene(sc, persistent=False)
    rb = sc["rigid"].copy()
    for step in range(4):
        s.set_bodies(rb)
        s.step(1)
        out = s.get_bodies()
        ref = run_scene_step("orc", as_world(dict(sc, rigid=rb)), dict(DEFAULT_PARAMS, persistent=False), steps=1)
        assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5, step
        assert np.abs(out["p"] - ref["p"]).max() <= 1e-6, step
        rb = out.copy()
    s.release()


def test_scene_100k_bodies_step_matches_oracle(cuda_device):
    """The single-large-scene workload at its full size (100k bodies in a 200 m box
    above the plane, initial overlaps allowed): after a short pre-roll, one frame
    from the same state against the oracle's frame."""
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world, large_scene
    from physx_gb300.world import DEFAULT_PARAMS
    sc = large_scene()
    s = Scene(sc, persistent=False)
    s.step(3)
    rb = s.get_bodies()
    s.step(1)
    out = s.get_bodies()
    st = s.stats()
    ref = run_scene_step("orc", as_world(dict(sc, rigid=rb)), dict(DEFAULT_PARAMS, persistent=False), steps=1)
    assert st["pairs"] > 100_000 and st["constraints"] > 1000
    assert np.isfinite(out["p"]).all()
    assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5
    assert np.abs(out["p"] - ref["p"]).max() <= 1e-6
    s.release()


def test_scene_stage_profiler_zones(cuda_device):
    """A frame of the large-scene step reports each stage as a profiler zone, in
    order, between the step's own zone (the reference's PX_PROFILE_ZONE protocol)."""
    import ctypes
    from physx_gb300 import lib
    from physx_gb300.scene import Scene
    L = lib()
    names = []
    START = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p)
    END = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p)
    s_cb = START(lambda n, d, c, u: names.append(n.decode()) or None)
    e_cb = END(lambda p, n, d, c, u: None)
    L.gbpx_set_profiler_callback.argtypes = [START, END, ctypes.c_void_p]
    s = Scene(_pile(135, 300))
    s.step(1)
    assert L.gbpx_set_profiler_callback(s_cb, e_cb, None) == 0
    try:
        s.step(1)
    finally:
        L.gbpx_set_profiler_callback(START(), END(), None)
    s.release()
    stages = [n for n in names if n.startswith("gbpx::scene::") and n != "gbpx::scene::step"]
    assert names[0] == "gbpx::scene::step"
    assert stages == ["gbpx::scene::broadphase", "gbpx::scene::narrowphase", "gbpx::scene::batching", "gbpx::scene::rows",
                      "gbpx::scene::iterations", "gbpx::scene::writeBack"], names


LARGE_TRACE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large_scene_trace.npz")


def test_scene_100k_bodies_600_steps_statistics_match_reference(cuda_device):
    """The single-large-scene workload over its full 600 steps (persistent pair
    state), against the reference's own 600-step trace (tests/golden/
    large_scene_trace.npz, made by tests/golden/make_large_trace.py with the
    reference build).  Bodies separate chaotically after a few hundred steps, so
    the check is on physical statistics, with these bounds:

    * kinetic energy within 1 % of the reference's at every one of the first 300
      steps (free fall and the first impacts), time-averaged within 2 %, peak within 1 %;
    * deepest ground penetration over the run at most 1.25 x the reference's + 1 cm;
      settled penetration (mean of the last 50 steps) within 3 cm of the reference's;
    * settled pile height (mean body height at the end) within 2 %;
    * fraction of bodies at rest at the end within 0.02."""
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import large_scene
    from trace_stats import FIELDS, body_checksum, step_stats
    ref = np.load(LARGE_TRACE)
    R = ref["stats"]
    assert list(ref["fields"]) == list(FIELDS)
    sc = large_scene()
    assert body_checksum(sc["rigid"]) == int(ref["checksum"]), "the workload generator changed"
    s = Scene(sc)
    rows = []
    for _ in range(int(ref["steps"])):
        s.step(1)
        st = step_stats(s.get_bodies(), sc["types"], sc["geoms"])
        rows.append([st[f] for f in FIELDS])
    s.release()
    G = np.array(rows)
    ke_r, ke_g = R[:, 0], G[:, 0]
    assert (np.abs(ke_g[:300] - ke_r[:300]) / ke_r[:300]).max() <= 0.01
    assert abs(ke_g.mean() - ke_r.mean()) <= 0.02 * ke_r.mean()
    assert abs(ke_g.max() - ke_r.max()) <= 0.01 * ke_r.max()
    assert -G[:, 1].min() <= 1.25 * -R[:, 1].min() + 0.01
    assert abs(G[-50:, 1].mean() - R[-50:, 1].mean()) <= 0.03
    assert abs(G[-1, 2] - R[-1, 2]) <= 0.02 * R[-1, 2]
    assert abs(G[-1, 4] - R[-1, 4]) <= 0.02
    assert np.isfinite(G).all()


@pytest.mark.parametrize("maker", ["pile", "hub"])
def test_scene_device_batching_equals_host_batching(cuda_device, maker):
    """PxBatchConstraintsTGS's rule run on the device (the parallel greedy colouring)
    and on the host give the same bytes frame after frame, persistent pair state
    on: a 3000-body pile (device path), and a scene with a body in more than 32
    constraints (the rule's second round: the device path hands the frame to the
    host)."""
    from physx_gb300.scene import Scene
    from scenarios import hub_scene
    sc = _pile(137, 3000) if maker == "pile" else hub_scene()
    a, b = Scene(sc), Scene(sc)
    b.set_device_batching(False)
    on_device = []
    for _ in range(12):
        a.step(1)
        b.step(1)
        on_device.append(a.batch_info()[1])
        assert a.get_bodies().tobytes() == b.get_bodies().tobytes()
        assert a.stats() == b.stats()
    if maker == "pile":
        assert all(on_device) and a.batch_info()[0] > 0
    a.release()
    b.release()
