"""The N-GPU path of bench.py on CPU: two gloo ranks (127.0.0.1) shard the
batched workload into independent scene sets (weak scaling, no data-path
collective) and reduce the whole-job figures: the slowest rank's time and the
bodies of all ranks."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    r, w, dist = bench.dist_setup(world)
    scenes = bench.rank_scenes(4, r, 16)
    bodies = int(scenes["body_count"].sum())
    ms = 10.0 + r                      # rank 1 is the slower one
    ms_all, bodies_all = bench.reduce_over_ranks(ms, bodies, dist)
    out.put((r, bodies, float(scenes["rigid"]["p"][:, 0].sum()), ms_all, bodies_all))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_and_reduction():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, b0, x0, ms0, tot0), (r1, b1, x1, ms1, tot1) = res
    assert (r0, r1) == (0, 1)
    assert x0 != x1                           # each rank has its own scenes
    assert ms0 == ms1 == 11.0                 # the slowest rank's time on every rank
    assert tot0 == tot1 == b0 + b1            # bodies of the whole job
    assert np.isfinite(x0) and b0 > 0 and b1 > 0


def test_world_size_must_match_gpus(monkeypatch):
    """--gpus N without N launched ranks is refused, not reported as N GPUs."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    with pytest.raises(SystemExit):
        bench.dist_setup(2)
    assert bench.dist_setup(1) == (0, 1, None)


def test_clock_sampler_names_this_ranks_gpu(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "3,GPU-abc")
    assert bench.smi_gpu_id(0) == "3" and bench.smi_gpu_id(1) == "GPU-abc"
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    assert bench.smi_gpu_id(2) == "2"
