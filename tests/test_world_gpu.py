"""Batched multi-scene world step on the GB300: each scene's frame against the
reference (golden fixture) and against the CPU oracle, determinism, graph
replay, error reporting."""
import numpy as np
import pytest

from oracle_libs import run_scene_step
from scenarios import batched_scenes, pile_scenes
from test_oracle_golden import (SCENE_FIXTURES, TGS_POSE_TOL, TGS_VEL_REL_TOL, load_scene_fixture, rigid_velocity,
                                velocity_error)

pytestmark = pytest.mark.gpu


def _world(scenes, **kw):
    from physx_gb300.world import World
    return World(scenes, **kw)


@pytest.mark.parametrize("path", SCENE_FIXTURES, ids=[p.rsplit("/", 1)[-1] for p in SCENE_FIXTURES])
def test_world_step_matches_reference_golden(cuda_device, path):
    scenes, ref = load_scene_fixture(path)
    w = _world(scenes)
    w.step(1)
    out = w.get_bodies()
    assert not w.status().any()
    assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= TGS_VEL_REL_TOL
    assert np.abs(out["p"] - ref["p"]).max() <= TGS_POSE_TOL and np.abs(out["q"] - ref["q"]).max() <= TGS_POSE_TOL
    w.release()


@pytest.mark.parametrize("shapes", [(0, 2), (0, 2, 3)])
def test_world_step_matches_oracle(cuda_device, shapes):
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = pile_scenes(71, 6, 40, shapes=shapes)
    w = _world(scenes)
    w.step(1)
    out = w.get_bodies()
    ref = run_scene_step("orc", scenes, DEFAULT_PARAMS, steps=1)
    # identical arithmetic except the integrator's sin/cos
    assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5
    assert np.abs(out["p"] - ref["p"]).max() <= 1e-6
    w.release()


def test_world_batched_workload_shape_and_determinism(cuda_device):
    """Scenes of 8..512 bodies dropped onto per-scene planes: 30 steps twice give
    identical states; graph replay equals direct launches; every body stays finite."""
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = batched_scenes(72, 96)
    a, b, c = _world(scenes), _world(scenes), _world(scenes)
    a.step(30, graph=True)
    b.step(30, graph=True)
    c.step(30, graph=False)
    ra, rb, rc = a.get_bodies(), b.get_bodies(), c.get_bodies()
    for f in ("linVel", "angVel", "q", "p"):
        assert np.array_equal(ra[f], rb[f]) and np.array_equal(ra[f], rc[f]), f
        assert np.isfinite(ra[f]).all()
    assert not a.status().any()
    # first step against the oracle on the same scenes
    d = _world(scenes)
    d.step(1)
    ref = run_scene_step("orc", scenes, DEFAULT_PARAMS, steps=1)
    out = d.get_bodies()
    assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5
    for w in (a, b, c, d):
        w.release()


def test_world_reports_pair_overflow(cuda_device):
    # 60 spheres packed into a ~1 m region overlap pairwise (~1770 pairs), far above
    # the 128 slots that one pair per body gives the scene
    scenes = pile_scenes(73, 2, 60, shapes=(0,), spread=1.0)
    w = _world(scenes, pairs_per_body=1)
    w.step(1)
    st = w.status()
    assert (st & 1).any()
    w.release()


def test_world_step_checked_retries_with_more_pair_slots(cuda_device):
    """Host retry with a larger arena: a step that overflows the pair slots is taken
    again from the bodies before it in a world with twice the slots per body until
    it fits; the result equals a world created with those slots."""
    scenes = pile_scenes(73, 2, 60, shapes=(0,), spread=1.0)
    w = _world(scenes, pairs_per_body=1)
    ppb = w.step_checked(2)
    assert ppb >= 16 and not w.status().any()
    ref = _world(scenes, pairs_per_body=ppb)
    ref.step(2, graph=False)
    assert w.get_bodies().tobytes() == ref.get_bodies().tobytes()
    w.release()
    ref.release()


def test_world_rejects_bad_input(cuda_device):
    from physx_gb300 import GbpxError
    scenes = pile_scenes(74, 1, 8, shapes=(0,))
    bad = dict(scenes)
    bad["types"] = scenes["types"].copy()
    bad["types"][0] = 1   # dynamic plane
    with pytest.raises(GbpxError):
        _world(bad)


def test_world_multi_round_batching_matches_oracle(cuda_device):
    """A body in more than 32 constraints: the second round of partitions and the
    static constraint's placement after it follow the reference's rule."""
    from physx_gb300.world import DEFAULT_PARAMS
    from scenarios import hub_scene
    scene = hub_scene()
    w = _world(scene)
    w.step(1)
    out = w.get_bodies()
    assert not w.status().any()
    ref = run_scene_step("orc", scene, DEFAULT_PARAMS, steps=1)
    assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5
    assert np.abs(out["p"] - ref["p"]).max() <= 1e-6
    w.release()


def test_world_persistent_steps_match_oracle(cuda_device):
    """Persistent mode (contact manifolds and friction patches kept between steps,
    the reference snippet's default) against the oracle's persistent frames, step
    by step over 10 steps of mixed piles.  The oracle's bodies are set to the
    world's after every step (the pair state stays each side's own), so last-ulp
    differences of sin/cos in the integration cannot grow over steps."""
    from oracle_libs import PersistentScenes
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = pile_scenes(75, 6, 40)
    w = _world(scenes)
    orc = PersistentScenes("orc", scenes, DEFAULT_PARAMS)
    for step in range(10):
        w.step(1)
        out = w.get_bodies()
        ref = orc.step().copy()
        orc.rb[:] = out
        assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5, step
        assert np.abs(out["p"] - ref["p"]).max() <= 1e-6, step
    assert not w.status().any()
    orc.release()
    w.release()


def test_world_fresh_mode_steps_match_oracle(cuda_device):
    """Persistence off: every step uses fresh caches and friction data, as the oracle's
    stateless frame does."""
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = pile_scenes(76, 6, 40)
    w = _world(scenes, persistent=False)
    rb = scenes["rigid"].copy()
    for step in range(6):
        # each step from the same input state (the per-step bar; trajectories of a
        # pile separate at the rounding level over many steps)
        w.set_bodies(rb)
        w.step(1)
        out = w.get_bodies()
        ref = run_scene_step("orc", dict(scenes, rigid=rb), DEFAULT_PARAMS, steps=1)
        assert velocity_error(rigid_velocity(ref), rigid_velocity(out)) <= 1e-5, step
        assert np.abs(out["p"] - ref["p"]).max() <= 1e-6, step
        rb = ref
    w.release()


@pytest.mark.parametrize("persistent", [True, False])
def test_world_block_per_scene_equals_warp_per_scene(cuda_device, persistent):
    """The scene stages run one warp per scene or one block per scene (large
    scenes); the arithmetic is the same, so both give the same bytes."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(141, 24, nmin=64, nmax=1500)
    a = World(scenes, persistent=persistent)
    b = World(scenes, persistent=persistent)
    a.set_large_bodies(1 << 30)   # every scene one warp
    b.set_large_bodies(0)         # every scene one block
    for step in range(40):
        a.step(1)
        b.step(1)
        if step % 8 == 7:
            assert a.get_bodies().tobytes() == b.get_bodies().tobytes(), step
    assert not a.status().any() and not b.status().any()
    assert a.stats()["constraints"] > 1000
    a.release()
    b.release()


def test_world_large_scenes_equal_scene_step(cuda_device):
    """Scenes above the block-per-scene threshold in a world step exactly like the
    same scenes stepped alone by the large-scene path."""
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world
    from physx_gb300.world import World
    from scenarios import random_scene
    parts = [random_scene(150 + k, n) for k, n in enumerate((700, 1500, 2600))]
    merged = dict(body_count=np.array([len(p["types"]) for p in parts], np.uint32), static_count=np.ones(3, np.uint32),
                  rigid=np.concatenate([p["rigid"] for p in parts]), types=np.concatenate([p["types"] for p in parts]),
                  geoms=np.concatenate([p["geoms"] for p in parts]), friction=np.concatenate([p["friction"] for p in parts]),
                  static_poses=np.concatenate([p["static_poses"] for p in parts]), static_types=np.concatenate([p["static_types"] for p in parts]),
                  static_geoms=np.concatenate([p["static_geoms"] for p in parts]))
    w = World(merged)
    assert w.info()["large_bodies"] == 512
    singles = [Scene(p) for p in parts]
    for step in range(6):
        w.step(1)
        got = w.get_bodies()
        off = 0
        for s in singles:
            s.step(1)
            ref = s.get_bodies()
            assert got[off:off + len(ref)].tobytes() == ref.tobytes(), step
            off += len(ref)
    assert not w.status().any()
    for s in singles:
        s.release()
    w.release()


def test_world_autotune_picks_a_threshold_and_keeps_results(cuda_device):
    """The autotuner (keyed on the scene-size histogram) sets a block-per-scene
    threshold from its candidates; the world's results do not change with it, and
    a second world of the same histogram takes the cached choice."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(142, 64, nmin=16, nmax=2048)
    a, b = World(scenes), World(scenes)
    a.step(5)
    b.step(5)
    thr, ms = a.autotune(sample_scenes=32, steps=2)
    assert thr in (64, 128, 256, 512, 1024, 2048, 0xffffffff) and ms > 0
    assert a.info()["large_bodies"] == thr
    thr2, ms2 = b.autotune(sample_scenes=32, steps=2)
    assert thr2 == thr and ms2 == 0.0
    assert b.tuning() == a.tuning()   # the cached choice includes the occupancies
    t = a.tuning()
    assert t["prep_blocks_per_sm"] in (0, 2, 3, 4) and t["narrowphase_blocks_per_sm"] in (0, 1, 2, 3)
    assert t["resident_stream"] in (0, 1, 2)
    b.set_large_bodies(512)
    b.set_occupancy(0, 0)
    b.set_resident_stream(1)
    a.step(10)
    b.step(10)
    assert a.get_bodies().tobytes() == b.get_bodies().tobytes()
    a.release()
    b.release()


def test_world_occupancy_keeps_results(cuda_device):
    """The blocks per SM of the row preparation and the heavy narrowphase kernels
    and the streamed-row levels of the resident solve (what the autotuner
    chooses after the threshold and the solve) do not change any result."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(144, 96, nmin=16, nmax=1024)
    worlds = [World(scenes) for _ in range(6)]
    worlds[1].set_occupancy(2, 1)
    worlds[2].set_occupancy(4, 3)
    for w, d in zip(worlds[3:], (0, 2, 3)):
        w.set_resident_stream(d)
    for _ in range(15):
        for w in worlds:
            w.step(1)
    ref = worlds[0].get_bodies().tobytes()
    for w in worlds:
        assert w.get_bodies().tobytes() == ref
        assert not w.status().any()
    for w in worlds:
        w.release()


def test_world_solve_staging_variants_equal(cuda_device):
    """The resident solve (variant 8: rows and velocities on chip for all
    iterations) and the warp-per-scene solve, which stages rows in 512 or 256 bytes
    per lane or uses them in place, with the body velocities in shared memory or
    in HBM: the nine variants give the same bytes."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(143, 48, nmin=16, nmax=500)
    worlds = [World(scenes) for _ in range(9)]
    for v, w in enumerate(worlds):
        w.set_solve_variant(v)
    for step in range(20):
        for w in worlds:
            w.step(1)
    ref = worlds[8].get_bodies().tobytes()
    for w in worlds:
        assert w.get_bodies().tobytes() == ref
        assert not w.status().any()
    for w in worlds:
        w.release()


def test_world_resident_solve_of_scenes_beyond_the_workspace(cuda_device):
    """Scenes whose rows (and, above about 4500 solver bodies, velocities) do not fit
    the resident solve's shared memory are solved with them in HBM: the same bytes
    as the block-per-scene solve, persistent pair state on."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(147, 6, nmin=1500, nmax=6000)
    assert scenes["body_count"].max() > 5000     # velocities of 5000+ bodies exceed the workspace
    a, b = World(scenes), World(scenes)
    a.set_solve_variant(8)
    b.set_solve_variant(2)
    for _ in range(90):
        a.step(1)
        b.step(1)
    prof = a.solve_profile()
    assert prof[:, 2].max() > 232448          # some scene's rows exceed the largest workspace
    assert a.get_bodies().tobytes() == b.get_bodies().tobytes()
    assert not a.status().any() and not b.status().any()
    a.release()
    b.release()


def test_world_full_size_batched_step_matches_oracle_sample(cuda_device):
    """The batched workload at its full size (4096 scenes, log-uniform [8,512]
    bodies, about 0.5M bodies) after a pre-roll: one step of the whole world
    against the oracle's step of 48 scenes sampled across the size range, from the
    same state (fresh caches, so the oracle's stateless frame applies)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import split_scenes
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = batched_scenes(4, 4096)
    w = _world(scenes, persistent=False)
    w.step(40)
    state = w.get_bodies()
    w.step(1)
    out = w.get_bodies()
    assert not w.status().any()
    counts = scenes["body_count"].astype(np.int64)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    idx = np.argsort(counts)[np.linspace(0, len(counts) - 1, 48).astype(np.int64)]
    sample = split_scenes(dict(scenes, rigid=state), idx)
    ref = run_scene_step("orc", sample, dict(DEFAULT_PARAMS, persistent=False), steps=1)
    got = np.concatenate([out[starts[i]:starts[i] + counts[i]] for i in idx])
    assert velocity_error(rigid_velocity(ref), rigid_velocity(got)) <= 1e-5
    assert np.abs(got["p"] - ref["p"]).max() <= 1e-6
    w.release()


def test_world_full_size_persistent_steps_match_oracle_sample(cuda_device):
    """The benchmarked configuration at full size: 4096 scenes (log-uniform [8,512]
    bodies, about 0.5M), persistent pair state, graph-replayed steps, resident
    solve.  A 48-scene size-stratified sample is stepped by the oracle's persistent
    frame in lockstep (each side keeps its own contact caches and friction data;
    the oracle's bodies are set to the world's after every step, so last-ulp sin/cos
    differences cannot grow); after 40 steps of pre-roll, 3 consecutive steps are
    held to the per-step bar (velocities 1e-5 relative, poses 1e-6)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import split_scenes
    from oracle_libs import PersistentScenes
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import DEFAULT_PARAMS
    scenes = batched_scenes(4, 4096)
    w = _world(scenes)
    counts = scenes["body_count"].astype(np.int64)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    idx = np.argsort(counts)[np.linspace(0, len(counts) - 1, 48).astype(np.int64)]
    sel = np.concatenate([np.arange(starts[i], starts[i] + counts[i]) for i in idx])
    orc = PersistentScenes("orc", split_scenes(scenes, idx), DEFAULT_PARAMS)
    for step in range(43):
        w.step(1, graph=True)
        out = w.get_bodies()
        got = out[sel]
        ref = orc.step().copy()
        orc.rb[:] = got
        if step >= 40:
            assert velocity_error(rigid_velocity(ref), rigid_velocity(got)) <= 1e-5, step
            assert np.abs(got["p"] - ref["p"]).max() <= 1e-6, step
            assert np.abs(got["q"] - ref["q"]).max() <= 1e-6, step
    assert not w.status().any()
    orc.release()
    w.release()


def test_world_step_host_equals_device_steps(cuda_device):
    """The end-to-end call (gbpx_world_step_host: bodies uploaded from pinned host
    memory, one graph-replayed step, bodies downloaded) gives the bytes of a
    device-resident step from the same state, step after step."""
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(151, 64, nmin=8, nmax=256)
    a, b = World(scenes), World(scenes)
    a.step(20)
    b.step(20)
    host_in, host_out = b.pinned_bodies(), b.pinned_bodies()
    host_out[:] = b.get_bodies()
    for _ in range(5):
        a.step(1)
        host_in[:] = host_out
        ms = b.step_host(host_in, host_out, 1)
        assert ms > 0
        assert host_out.tobytes() == a.get_bodies().tobytes()
    assert not a.status().any() and not b.status().any()
    a.release()
    b.release()
