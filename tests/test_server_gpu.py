"""Serving pool (continuous batching over resident scenes): a scene's result is the
same served alone, served in a mix of other scenes' requests, and stepped by the
batched world; admission respects the slot budget; retirement waits for owed steps."""
import numpy as np
import pytest

from scenarios import pile_scenes

pytestmark = pytest.mark.gpu


def one_scene(scenes, k):
    counts = scenes["body_count"].astype(np.int64)
    b0 = int(counts[:k].sum())
    sl = slice(b0, b0 + int(counts[k]))
    return dict(rigid=scenes["rigid"][sl].copy(), types=scenes["types"][sl], geoms=scenes["geoms"][sl], friction=scenes["friction"][sl],
                static_poses=scenes["static_poses"][k:k + 1], static_types=scenes["static_types"][k:k + 1],
                static_geoms=scenes["static_geoms"][k:k + 1], body_count=np.array([counts[k]], np.uint32),
                static_count=np.ones(1, np.uint32))


def test_scene_result_same_alone_and_in_mix(cuda_device):
    from physx_gb300.server import Server
    from physx_gb300.world import World
    scenes = pile_scenes(81, 5, 40, shapes=(0, 2, 3))
    parts = [one_scene(scenes, k) for k in range(5)]
    # served alone: 10 steps in one request
    s1 = Server([64], [2])
    a = s1.admit(parts[0])
    s1.submit(a, 10, 1)
    tags, lat = s1.drain()
    assert list(tags) == [1] and (lat >= 0).all()
    alone = s1.read_scene(a)
    s1.release()
    # served in a mix: the same 10 steps as three requests, interleaved with other scenes' requests
    s2 = Server([64], [8])
    ids = [s2.admit(p) for p in parts]
    rng = np.random.default_rng(0)
    tag = 100
    for chunk in (3, 3, 4):
        s2.submit(ids[0], chunk, tag)
        tag += 1
        for other in ids[1:]:
            s2.submit(other, int(rng.integers(1, 5)), tag)
            tag += 1
        s2.pump()
    tags, lat = s2.drain()
    assert sorted(tags) == list(range(100, tag))
    mixed = s2.read_scene(ids[0])
    s2.release()
    assert np.array_equal(alone.view(np.uint8), mixed.view(np.uint8))
    # the batched world gives the same bodies
    w = World(parts[0])
    w.step(10)
    ref = w.get_bodies()
    w.release()
    assert np.array_equal(alone.view(np.uint8), ref.view(np.uint8))


def test_admission_budget_and_retirement(cuda_device):
    from physx_gb300 import GBPX_OK, GbpxError  # noqa: F401
    from physx_gb300.server import Server
    scenes = pile_scenes(82, 4, 20, shapes=(0,))
    parts = [one_scene(scenes, k) for k in range(4)]
    s = Server([32], [2])
    a = s.admit(parts[0])
    s.admit(parts[1])
    with pytest.raises(GbpxError) as e:
        s.admit(parts[2])
    assert e.value.code == -6   # GBPX_ERR_BUDGET: no free slot
    s.submit(a, 5, 7)
    with pytest.raises(GbpxError):
        s.retire(a)            # owes steps
    tags, _ = s.drain()
    assert list(tags) == [7]
    s.retire(a)
    s.admit(parts[3])          # the slot is free again
    assert s.stats()["live"] == 2
    s.release()


def test_scene_result_same_with_lanes_and_classes(cuda_device):
    """Scenes of several body-count classes, each class split into two lanes, served
    in a mix of requests: every scene's bodies equal the batched world's after the
    same number of steps."""
    from physx_gb300.server import Server
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import World
    scenes = batched_scenes(83, 6, nmin=20, nmax=200)
    parts = [one_scene(scenes, k) for k in range(6)]
    s = Server([32, 64, 128, 256], [2, 2, 2, 2], lanes_per_class=2)
    ids = [s.admit(p) for p in parts]
    rng = np.random.default_rng(1)
    owed = [0] * len(ids)
    tag = 0
    for _ in range(4):
        for k, sid in enumerate(ids):
            n = int(rng.integers(1, 4))
            s.submit(sid, n, tag)
            owed[k] += n
            tag += 1
        s.pump()
    tags, _ = s.drain()
    assert sorted(tags) == list(range(tag))
    for k, sid in enumerate(ids):
        got = s.read_scene(sid)
        w = World(parts[k])
        w.step(owed[k])
        assert np.array_equal(got.view(np.uint8), w.get_bodies().view(np.uint8)), k
        w.release()
    s.release()


def test_native_poisson_load_retires_and_readmits(cuda_device):
    """The open-loop load run in the library (gbpx_server_run_load): requests
    complete, scenes that reach their lifetime are retired and replaced, and the
    figures are consistent."""
    from physx_gb300.serve_load import run_poisson
    r = run_poisson(duration=2.0, rate=3000.0, budget_bytes=2e9, nmin=16, nmax=256, life=(5, 30), seed=9, per_class=3, lanes_per_class=2)
    assert r["completed"] > 1000 and r["completed"] <= r["submitted"]
    assert r["retired"] > 0 and r["admitted_after_start"] > 0
    assert r["body_steps_per_s"] > 0 and r["p50_ms"] > 0 and r["p99_ms"] >= r["p50_ms"]
    assert r["lanes"] == 2 * len(r["classes"])


def test_snapshot_and_restore_continue_the_scene(cuda_device):
    """Eviction and re-admission: a scene snapshotted after 12 steps, retired and
    restored into another slot, then stepped 10 more times, ends with the bytes of
    the same scene stepped 22 times without interruption; the snapshot carries its
    pair list with the contact manifolds and friction patches."""
    from physx_gb300.server import Server
    scenes = pile_scenes(83, 3, 40, shapes=(0, 2, 3))
    part = one_scene(scenes, 0)
    s = Server([64], [4])
    ref = s.admit(part)
    a = s.admit(part)
    s.submit(ref, 22, 1)
    s.submit(a, 12, 2)
    s.drain()
    snap = s.snapshot(a)
    nb, ns, npairs, pair_state = np.frombuffer(snap[8:24].tobytes(), np.uint32)
    assert nb == len(part["rigid"]) and ns == 1 and npairs > 0 and pair_state == 1
    s.retire(a)
    s.admit(one_scene(scenes, 1))   # takes the freed slot
    b = s.restore(snap)
    assert b != a
    s.submit(b, 10, 3)
    s.drain()
    assert s.read_scene(b).tobytes() == s.read_scene(ref).tobytes()
    from physx_gb300 import GbpxError
    with pytest.raises(GbpxError):
        s.restore(snap[:-4])   # a truncated snapshot is refused
    s.release()
