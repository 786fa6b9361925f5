"""Benchmark of the batched rigid-body step on GB300.

Workload: 4096 independent scenes, body counts log-uniform in [8, 512] (sphere /
box / capsule mix), dropped from U(1, 20) m onto a per-scene ground plane; TGS
4 position / 1 velocity iterations, dt = 1/60 s, FP32 (synthetic, seeded).
A step is one frame of every scene: bounds, ABP broadphase, contacts, TGS
batching / rows / solve / integration, all in one persistent launch.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput in
body-steps/s; `e2e` re-measures it through the public world API with the
bodies uploaded from and downloaded to pinned host memory every step.
`--impl reference` times the CPU restatement of the reference path (the
oracle) on all host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s batched+served vs plain GPU step at 1e-5 tol; p50/p99 latency"
UNIT = "body-steps/s"
WORKLOAD = ("batched: 4096 scenes, bodies log-uniform [8,512] sphere/box/capsule, drop U(1,20) m onto per-scene plane, "
            "ABP + contacts + TGS 4/1, dt 1/60, FP32")


SOLVE_VARIANTS = ["warp per scene, rows in place, velocities on chip", "warp per scene, 256 B staging per lane, velocities on chip",
                  "warp per scene, 512 B staging per lane, velocities on chip", "warp per scene, rows in place, velocities in HBM",
                  "warp per scene, 256 B staging per lane, velocities in HBM", "warp per scene, 512 B staging per lane, velocities in HBM",
                  "warp per scene, 400 B staging per lane, velocities on chip", "warp per scene, 400 B staging per lane, velocities in HBM",
                  "resident: velocities on chip; rows bulk-copied on chip once, or streamed through a two-slot ring"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbpx", choices=["gbpx", "reference"])
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--preroll", type=int, default=120, help="untimed steps first, so bodies have landed (contact-rich state)")
    ap.add_argument("--cpu-scenes", type=int, default=1024, help="scenes in the bounded CPU-baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--plain-scenes", type=int, default=256, help="scenes timed one-per-launch for the plain comparison")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="duration of the Poisson serving run (0 = skip)")
    ap.add_argument("--serve-lanes", type=int, default=1, help="lanes per body-count class of the serving pool")
    ap.add_argument("--serve-rate", type=float, default=20000.0, help="request arrivals per second")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="HBM budget of the serving pool")
    ap.add_argument("--extras", type=int, default=1, help="also measure the pyramid, 1M-AABB broadphase and 100k-body scene workloads")
    ap.add_argument("--pyramid-steps", type=int, default=300)
    ap.add_argument("--bp-frames", type=int, default=10)
    ap.add_argument("--bp-cpu-frames", type=int, default=1)
    ap.add_argument("--large-steps", type=int, default=600, help="frames of the 100k-body single-scene run")
    ap.add_argument("--large-cpu-frames", type=int, default=1)
    ap.add_argument("--large-bodies", type=int, default=0,
                    help="block-per-scene threshold of the world's scene stages (0 = autotuned for the scene-size histogram)")
    ap.add_argument("--joint-frames", type=int, default=20)
    ap.add_argument("--profile-extra", default="", choices=["", "broadphase", "large-scene", "joints", "convex-core", "pgs"],
                    help="only run one frame of this side workload inside a profiler range and exit")
    ap.add_argument("--profile-step", type=int, default=0,
                    help="only build the state (pre-roll, autotune, warm-up), then run this many un-captured steps inside a "
                         "profiler range (for ncu --profile-from-start off) and exit")
    return ap.parse_args()


# ---------------------------------------------------------------- CPU baseline (oracle restatement, all cores)
def _cpu_proc(scenes, pv, it, preroll, warmup, steps, barrier, out):
    """One host process of the CPU baseline: its scenes through the oracle's
    persistent frame (contact caches and friction data kept between steps, one
    handle for the whole run), `preroll` + `warmup` untimed steps, then `steps`
    timed steps between barriers shared with the other processes."""
    import ctypes
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import _p, oracle
    L = oracle()
    keep = [np.ascontiguousarray(scenes[k], d) for k, d in (("body_count", np.uint32), ("static_count", np.uint32), ("types", np.int32),
                                                              ("geoms", np.float32), ("friction", np.float32), ("static_poses", np.float32),
                                                              ("static_types", np.int32), ("static_geoms", np.float32))]
    rb = np.ascontiguousarray(scenes["rigid"]).copy()
    L.orc_persistent_create.restype = ctypes.c_void_p
    h = ctypes.c_void_p(L.orc_persistent_create())

    def step():
        L.orc_scene_step_persistent(h, ctypes.c_uint32(len(keep[0])), _p(keep[0]), _p(keep[1]), _p(rb), _p(keep[2]), _p(keep[3]),
                                    _p(keep[4]), _p(keep[5]), _p(keep[6]), _p(keep[7]), _p(pv), _p(it))

    for _ in range(preroll + warmup):
        step()
    barrier.wait()
    t0 = time.monotonic()
    for _ in range(steps):
        step()
    t1 = time.monotonic()
    barrier.wait()
    L.orc_persistent_release(h)
    out.put((t0, t1, int(keep[0].sum())))


def split_scenes(scenes, idx):
    import numpy as np
    counts = scenes["body_count"].astype(np.int64)
    starts = np.zeros(len(counts), np.int64)
    starts[1:] = np.cumsum(counts)[:-1]
    sel = np.concatenate([np.arange(starts[i], starts[i] + counts[i]) for i in idx]) if len(idx) else np.zeros(0, np.int64)
    return dict(body_count=counts[idx], static_count=scenes["static_count"][idx], rigid=scenes["rigid"][sel], types=scenes["types"][sel],
                geoms=scenes["geoms"][sel], friction=scenes["friction"][sel], static_poses=scenes["static_poses"][idx],
                static_types=scenes["static_types"][idx], static_geoms=scenes["static_geoms"][idx])


def cpu_sample(nb_scenes_total, nb_sample):
    """The CPU sample: every k-th scene of the world, an even spread of scene sizes."""
    import numpy as np
    return np.linspace(0, nb_scenes_total - 1, min(nb_sample, nb_scenes_total)).astype(np.int64)


def cpu_baseline(scenes, params, nb_scenes, steps, cores, preroll=0, warmup=1, ctx=None):
    """The oracle restatement of the reference frame on a bounded sample of the
    scenes, split across `cores` host processes (spawned), persistent pair state
    as the world runs: each process pre-rolls `preroll` steps and warms up
    `warmup` steps, then all time `steps` consecutive steps together; the wall
    time is from the first process's start to the last one's end."""
    import multiprocessing as mp
    from physx_gb300.world import param_vector
    pv, it = param_vector(params)
    S = len(scenes["body_count"])
    idx = cpu_sample(S, nb_scenes)
    chunks = [c for c in (idx[i::cores] for i in range(cores)) if len(c)]
    ctx = ctx or mp.get_context("spawn")
    barrier = ctx.Barrier(len(chunks))
    q = ctx.Queue()
    procs = [ctx.Process(target=_cpu_proc, args=(split_scenes(scenes, c), pv, it, preroll, warmup, steps, barrier, q)) for c in chunks]
    for p in procs:
        p.start()
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
        if p.exitcode != 0:
            raise RuntimeError("CPU baseline process failed (exit code %s)" % p.exitcode)
    wall = max(r[1] for r in res) - min(r[0] for r in res)
    bodies = sum(r[2] for r in res)
    return dict(value=bodies * steps / wall, unit=UNIT, cores=len(chunks), kind="port",
                sample="%d of %d scenes (%d bodies, every %d-th by index), %d pre-roll + %d warm-up + %d timed persistent steps, "
                       "oracle restatement, %d processes" % (len(idx), S, bodies, max(1, S // max(1, len(idx))), preroll, warmup, steps, len(chunks)),
                seconds=wall, ms_per_step=1000.0 * wall / steps)


# ---------------------------------------------------------------- clocks
def smi_gpu_id(local_rank):
    """This rank's GPU as nvidia-smi names it: the LOCAL_RANK-th entry of
    CUDA_VISIBLE_DEVICES (an index or a UUID) when that is set, else LOCAL_RANK."""
    vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    return vis[local_rank] if local_rank < len(vis) else str(local_rank)


class ClockSampler:
    """nvidia-smi samples of this rank's GPU (only) during the timed region."""

    def __init__(self, gpu="0"):
        self.samples = []
        self.proc = None
        self.gpu = gpu

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                                          "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                                          "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = sorted(float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit())
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 3 + k and s[3 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(stage):
    """DRAM bytes (read + write) per launch of a stage's kernel on the bench workload, from the
    committed ncu summary (profiles/dram_traffic_world_step.txt, lines `<stage>: <bytes>`), if present."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_world_step.txt")
    try:
        for line in open(path):
            if line.startswith(stage + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def bench_pyramid(steps):
    """The 210-box pyramid of the reference's immediate-mode snippet (one scene, the world
    API), against the oracle restatement of the same frame on one host thread."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import PersistentScenes
    from physx_gb300.workloads import pyramid_scene
    from physx_gb300.world import DEFAULT_PARAMS, World
    sc = pyramid_scene()
    w = World(sc)
    w.step(3, graph=True)
    w.synchronize()
    ms = w.time_steps(steps, graph=True)
    w.release()
    ps = PersistentScenes("orc", sc, DEFAULT_PARAMS)
    t = time.perf_counter()
    ps.step(steps)
    cpu_s = time.perf_counter() - t
    ps.release()
    n = len(sc["rigid"])
    return dict(workload="210-box pyramid (20 levels, h 0.5, jitter 0.01 m / 2 deg), plane, TGS 4/1, dt 1/60", bodies=n, steps=steps,
                ms_per_step=ms / steps, value=n * steps / (ms / 1000.0), unit=UNIT,
                cpu_baseline=dict(value=n * steps / cpu_s, unit=UNIT, cores=1, kind="port",
                                  sample="the same %d steps, oracle restatement, one thread" % steps))


def bench_broadphase(frames, cpu_frames):
    """1M AABBs, 10% moved per frame: PxBroadPhase (eABP) update + fetchResults through the
    C ABI with host arrays, per frame; the oracle ABP restatement on one host thread."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import CpuBroadPhase
    from physx_gb300.broadphase import BroadPhase
    from physx_gb300.workloads import aabb_stress_frames

    def algorithmic(fr, n_total, active, created, lost):
        return 36 * len(fr["updated"]) + 28 * n_total + 16 * active + 8 * (created + lost)

    bp = BroadPhase()
    times, pairs, byts, dev_ms, host_ms = [], [], [], [], []
    for f, fr in enumerate(aabb_stress_frames(frames=frames + 1)):
        t = time.perf_counter()
        bp.update(fr["created"], fr["updated"], fr["removed"], fr["bounds"], fr["groups"], fr["distances"], fr["capacity"])
        c, l = bp.fetch_results()
        dt = time.perf_counter() - t
        st = bp.stats()
        if f == 0:
            continue   # the first frame creates every box
        hm, dm = bp.timing()
        host_ms.append(hm)
        dev_ms.append(dm)
        times.append(dt)
        pairs.append(st["active"] + len(c) + len(l))
        byts.append(algorithmic(fr, st["live"], st["active"], len(c), len(l)))
    bp.release()
    ms = 1000.0 * float(np.median(times))
    k = int(np.argsort(times)[len(times) // 2])
    cpu = CpuBroadPhase("orc")
    ct = []
    for f, fr in enumerate(aabb_stress_frames(frames=cpu_frames + 1)):
        t = time.perf_counter()
        cpu.update(fr)
        if f:
            ct.append(time.perf_counter() - t)
    cpu.release()
    cpu_ms = 1000.0 * float(np.median(ct))
    return dict(workload="1M AABBs U(0,1000)^3, half-extents lognormal(ln 0.5, 0.5), all dynamic, distance 0; 10% moved N(0, 0.2 m) per frame",
                frames=frames, ms_per_frame=ms, value=pairs[k] / (ms / 1000.0), unit="pairs/s (active + created + lost)",
                device_ms_per_frame=float(np.median(dev_ms)), host_staging_ms_per_frame=float(np.median(host_ms)),
                e2e_note="host arrays in, created/lost pairs out (PxBroadPhase::update + fetchResults)",
                algorithmic_gbs=byts[k] / (ms / 1000.0) / 1e9,
                cpu_baseline=dict(value=pairs[k] / (cpu_ms / 1000.0), ms_per_frame=cpu_ms, unit="pairs/s", cores=1, kind="port",
                                  sample="%d frames, oracle ABP restatement, one thread" % cpu_frames))


def bench_large_scene(steps, cpu_frames):
    """Single large scene: 100k sphere/box/capsule bodies in a 200 m box above the
    plane, the full `steps`-frame run through gbpx_scene_* (persistent pair state),
    then end to end through host memory, and the oracle's persistent frame of the
    final state on one host thread."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import PersistentScenes
    from physx_gb300.scene import Scene
    from physx_gb300.workloads import as_world, large_scene
    from physx_gb300.world import DEFAULT_PARAMS
    sc = large_scene()
    n = len(sc["rigid"])
    s = Scene(sc)
    total, stages, chunks, last = 0.0, {}, 0, None
    for done in range(0, steps, 50):
        k = min(50, steps - done)
        ms, st = s.time_steps(k)
        total += ms * k
        chunks += 1
        last = (ms, st, dict(s.stats(), batching_passes=s.batch_info()[0], batched_on_device=s.batch_info()[1]))
    ms_step = total / steps
    tail_ms, tail_stages, tail_stats = last
    state = s.get_bodies()
    # end to end: bodies from pinned-free host arrays in and out every frame
    host_in, host_out = state.copy(), np.empty_like(state)
    e2e_frames = 10
    e2e_ms = 0.0
    for _ in range(e2e_frames):
        e2e_ms += s.step_host(host_in, host_out, 1)
        host_in[:] = host_out
    s.release()
    ps = PersistentScenes("orc", as_world(dict(sc, rigid=state)), DEFAULT_PARAMS)
    ps.step(1)   # the first oracle frame builds the pair caches
    t = time.perf_counter()
    ps.step(cpu_frames)
    cpu_s = (time.perf_counter() - t) / cpu_frames
    ps.release()
    return dict(workload="one scene of 100k bodies (1/3 spheres r U(0.25,1), 1/3 boxes h U(0.25,1)^3, 1/3 capsules r U(0.2,0.5) hh U(0.25,1)), "
                         "positions U([-100,100]x[0,200]x[-100,100]) m, random orientations, plane y=0, ABP + contacts + TGS 4/1, dt 1/60",
                bodies=n, steps=steps, ms_per_step=ms_step, value=n / (ms_step / 1000.0), unit=UNIT,
                last_50_steps=dict(ms_per_step=tail_ms, stages_ms=tail_stages, **tail_stats),
                e2e=dict(value=n * e2e_frames / (e2e_ms / 1000.0), unit=UNIT, h2d_bytes_per_step=n * 96, d2h_bytes_per_step=n * 96),
                cpu_baseline=dict(value=n / cpu_s, unit=UNIT, cores=1, kind="port",
                                  sample="%d persistent frame(s) of the final state, oracle restatement, one thread" % cpu_frames))


def joint_workload(chains=1500):
    """The joint bench frame: `chains` chains of 2-9 boxes hung from static
    anchors by spherical / revolute / fixed / prismatic / sprung joints (rows
    written from the poses, as a joint shader would), the frame after one
    settling frame."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from joint_scenes import joint_frame, make_joint_scene
    from oracle_libs import advance_rigid, run_joints
    sc = make_joint_scene(77, nb_chains=chains, links=(2, 9))
    fr = joint_frame(sc, sc["rigid"])
    r = run_joints("orc", fr)
    return joint_frame(sc, advance_rigid(sc["rigid"], r["vel"], r["pose"]))


def bench_joints(frames, cpu_frames):
    """Joints (PxCreateJointConstraintsTGS + PxSolveConstraintsTGS, 4 position +
    1 velocity iterations) through gbpx_joint_frame with host arrays in and out,
    against the oracle's frame on one host thread."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import run_joints
    from physx_gb300.solver import joint_frame as gpu_joint_frame
    fr = joint_workload()
    nj, nrows = len(fr["joint_a"]), len(fr["rows"])
    for _ in range(3):
        gpu_joint_frame(fr)
    times = []
    for _ in range(frames):
        t = time.perf_counter()
        out = gpu_joint_frame(fr)
        times.append(time.perf_counter() - t)
    ms = 1000.0 * float(np.median(times))
    t = time.perf_counter()
    for _ in range(cpu_frames):
        run_joints("orc", fr)
    cpu_ms = 1000.0 * (time.perf_counter() - t) / cpu_frames
    types = np.bincount(out["header_type"], minlength=9)
    return dict(workload="%d joints (%d rows) in 1500 chains of 2-9 boxes hung from static anchors: spherical / revolute / fixed / "
                         "prismatic / sprung joints with limits, drives, restitution, break forces" % (nj, nrows),
                joints=nj, rows=nrows, bodies=int(fr["nb_dyn"]), headers_per_pair_path=int(types[2]), headers_4_wide=int(types[8]),
                frames=frames, ms_per_frame=ms, value=nj / (ms / 1000.0), unit="joints/s (one TGS frame each)",
                e2e_note="host arrays in (bodies, rows, parameters), velocities, poses and impulses out, every frame",
                cpu_baseline=dict(value=nj / (cpu_ms / 1000.0), ms_per_frame=cpu_ms, unit="joints/s", cores=1, kind="port",
                                  sample="%d frame(s) of the same state, oracle restatement, one thread" % cpu_frames))


def pgs_workload(copies=48, spacing=3.0, friction=0.5):
    """The immediate-mode snippet's 210-box pyramid repeated `copies` times side
    by side (z offsets of `spacing` m) in one PGS frame: contacts from the
    GB300 narrowphase for every box pair whose bounds (inflated by the contact
    distance) overlap and for every box against the plane."""
    import numpy as np
    from physx_gb300.contacts import generate_contacts
    from physx_gb300.workloads import pyramid_scene
    base = pyramid_scene()
    n0 = len(base["rigid"])
    rigid = np.concatenate([base["rigid"]] * copies)
    for k in range(copies):
        rigid["p"][k * n0:(k + 1) * n0, 2] += np.float32(spacing * k)
    n = len(rigid)
    half = float(base["geoms"][0, 0])
    r = half * 1.05 + 0.04
    A, B = [], []
    for k in range(copies):
        p = rigid["p"][k * n0:(k + 1) * n0].astype(np.float64)
        close = np.all(np.abs(p[:, None, :] - p[None, :, :]) <= 2 * r, axis=2)
        i, j = np.nonzero(np.triu(close, 1))
        A.append(i + k * n0)
        B.append(j + k * n0)
    A.append(np.arange(n))
    B.append(np.full(n, n))   # the plane, static body n
    A = np.concatenate(A).astype(np.uint32)
    B = np.concatenate(B).astype(np.uint32)
    box = np.array([half, half, half, 0], np.float32)
    plane_pose = base["static_poses"][0]
    pose = lambda idx: np.where((idx < n)[:, None], np.concatenate([rigid["q"], rigid["p"]], 1)[np.minimum(idx, n - 1)], plane_pose)  # noqa: E731
    pairs = dict(type0=np.full(len(A), 3, np.int32), geom0=np.tile(box, (len(A), 1)), type1=np.where(B < n, 3, 1).astype(np.int32),
                 geom1=np.where((B < n)[:, None], box, 0).astype(np.float32), pose0=pose(A).astype(np.float32), pose1=pose(B).astype(np.float32))
    cnt, out = generate_contacts(pairs, max_per_pair=4)
    keep = np.flatnonzero(cnt > 0)
    count = cnt[keep].astype(np.uint32)
    start = np.zeros(len(keep), np.uint32)
    start[1:] = np.cumsum(count)[:-1]
    contacts = np.ascontiguousarray(np.concatenate([out[k, :cnt[k]] for k in keep]), np.float32)
    mat = np.zeros((len(keep), 3), np.float32)
    mat[:, 0] = mat[:, 1] = friction
    return dict(rigid=rigid, static_poses=base["static_poses"], body_a=A[keep], body_b=B[keep], contact_start=start, contact_count=count,
                contacts=contacts, material=mat)


def bench_pgs(frames, cpu_frames):
    """One immediate-mode PGS frame (PxConstructSolverBodies, PxBatchConstraints,
    PxCreateContactConstraints, PxSolveConstraints 4/1, PxIntegrateSolverBodies)
    through gbpx_pgs_solve with host arrays in and out, per frame; the oracle's
    frame on one host thread."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import run_pgs
    from physx_gb300.solver import pgs_step
    w = pgs_workload()
    args = (w["rigid"], w["static_poses"], w["body_a"], w["body_b"], w["contact_start"], w["contact_count"], w["contacts"], w["material"])
    for _ in range(3):
        out = pgs_step(*args)
    times = []
    for _ in range(frames):
        t = time.perf_counter()
        out = pgs_step(*args)
        times.append(time.perf_counter() - t)
    ms = 1000.0 * float(np.median(times))
    sc = dict(types=np.zeros(len(w["rigid"]), np.int32), rigid=w["rigid"], static_poses=w["static_poses"])
    t = time.perf_counter()
    for _ in range(cpu_frames):
        run_pgs("orc", sc, *args[2:])
    cpu_ms = 1000.0 * (time.perf_counter() - t) / cpu_frames
    n, nc = len(w["rigid"]), len(w["body_a"])
    types = np.bincount(out["header_type"], minlength=8)
    return dict(workload="48 copies of the snippet's 210-box pyramid side by side (%d boxes, %d contact constraints, %d contacts), "
                         "plane, PGS 4 position / 1 velocity iterations, dt 1/60" % (n, nc, len(w["contacts"])),
                bodies=n, constraints=nc, headers_block=int(types[6] + types[7]), headers_per_pair=int(types[1] + types[5]),
                frames=frames, ms_per_frame=ms, value=n / (ms / 1000.0), unit="body-steps/s (one PGS frame each)",
                e2e_note="host arrays in (bodies, contacts, materials), velocities, poses and impulses out, every frame",
                cpu_baseline=dict(value=n / (cpu_ms / 1000.0), ms_per_frame=cpu_ms, unit="body-steps/s", cores=1, kind="port",
                                  sample="%d frame(s) of the same state, oracle restatement, one thread" % cpu_frames))


def convex_core_workload(reps=8, unique=32768):
    """Convex-core contact pairs (every core type against every shape type, 60 %
    axis-aligned for face contacts): `unique` seeded pairs repeated `reps` times
    (262,144 pairs, the no-allocation entry point's limit)."""
    import numpy as np
    from physx_gb300.workloads import convex_core_pairs
    base = convex_core_pairs(7, unique, aligned_frac=0.6)
    return {k: np.ascontiguousarray(np.concatenate([v] * reps)) for k, v in base.items()}


def bench_convex_core(iters, cpu_pairs):
    """Convex-core contact generation (PxGenerateContacts for PxConvexCoreGeometry
    pairs): device-resident through gbpx_generate_contacts_device_noalloc on the
    caller's device arrays (CUDA events on the launching stream, L2 flushed
    before every timed call), end to end through gbpx_generate_contacts with host
    arrays in and contacts out, and the oracle on one host thread."""
    import ctypes
    import numpy as np
    import torch
    import physx_gb300
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_libs import run_contacts
    from physx_gb300.contacts import generate_contacts
    pairs = convex_core_workload()
    n = len(pairs["type0"])
    L = physx_gb300.lib()
    f = L.gbpx_generate_contacts_device_noalloc
    f.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    dev = torch.device("cuda:0")
    keys = ("type0", "geom0", "type1", "geom1", "pose0", "pose1")
    ins = [torch.from_numpy(pairs[k]).to(dev) for k in keys]
    out = torch.zeros((n, 4, 8), dtype=torch.float32, device=dev)
    cnt = torch.zeros(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream()
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)   # 256 MB, twice the L2

    def launch():
        physx_gb300.check(f(*[t.data_ptr() for t in ins], n, 0.04, 1.0, out.data_ptr(), cnt.data_ptr(), ctypes.c_void_p(stream.cuda_stream)),
                          "gbpx_generate_contacts_device_noalloc")
    with torch.cuda.stream(stream):
        for _ in range(3):
            launch()
        times = []
        for _ in range(iters):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            launch()
            e1.record(stream)
            stream.synchronize()
            times.append(e0.elapsed_time(e1))
    dev_ms = float(np.median(times))
    counts = cnt.cpu().numpy()
    generate_contacts(pairs, max_per_pair=4)
    e2e = []
    for _ in range(iters):
        t = time.perf_counter()
        generate_contacts(pairs, max_per_pair=4)
        e2e.append(time.perf_counter() - t)
    e2e_ms = 1000.0 * float(np.median(e2e))
    sample = {k: v[:cpu_pairs] for k, v in pairs.items()}
    t = time.perf_counter()
    run_contacts("orc", sample, max_per_pair=4)
    cpu_s = time.perf_counter() - t
    return dict(workload="%d convex-core pairs (point / segment / box / ellipsoid / cylinder / cone cores with margins against spheres, "
                         "planes, capsules, boxes and convex cores; 32768 seeded pairs repeated 8 times)" % n,
                pairs=n, contacts=int(counts.sum()), pairs_with_contacts=int((counts > 0).sum()), face_pairs=int((counts > 1).sum()),
                device_ms=dev_ms, value=n / (dev_ms / 1000.0), unit="pairs/s",
                note="device-resident, 5 kernels per call (bucket count / offsets / scatter, two generators); L2 flushed before each call",
                e2e=dict(value=n / (e2e_ms / 1000.0), ms=e2e_ms, unit="pairs/s", h2d_bytes=int(n * 96), d2h_bytes=int(n * (4 + 128))),
                cpu_baseline=dict(value=cpu_pairs / cpu_s, unit="pairs/s", cores=1, kind="port",
                                  sample="first %d pairs, oracle restatement, one thread" % cpu_pairs))


def profile_extra(which):
    """One frame of a side workload inside a profiler range (for ncu
    --profile-from-start off), after untimed warm-up frames."""
    import physx_gb300
    L = physx_gb300.lib()
    if which == "broadphase":
        from physx_gb300.broadphase import BroadPhase
        from physx_gb300.workloads import aabb_stress_frames
        bp = BroadPhase()
        for f, fr in enumerate(aabb_stress_frames(frames=4)):
            if f == 3:
                physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
            bp.update(fr["created"], fr["updated"], fr["removed"], fr["bounds"], fr["groups"], fr["distances"], fr["capacity"])
            bp.fetch_results()
            if f == 3:
                physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        out = bp.stats()
        bp.release()
    elif which == "large-scene":
        from physx_gb300.scene import Scene
        from physx_gb300.workloads import large_scene
        s = Scene(large_scene())
        s.step(300)
        physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
        s.step(1)
        physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        out = s.stats()
        s.release()
    elif which == "pgs":
        from physx_gb300.solver import pgs_step
        w = pgs_workload()
        args = (w["rigid"], w["static_poses"], w["body_a"], w["body_b"], w["contact_start"], w["contact_count"], w["contacts"], w["material"])
        pgs_step(*args)
        physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
        r = pgs_step(*args)
        physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        out = dict(bodies=len(w["rigid"]), constraints=len(w["body_a"]), headers=len(r["header_start"]))
    elif which == "convex-core":
        from physx_gb300.contacts import generate_contacts
        pairs = convex_core_workload()
        generate_contacts(pairs, max_per_pair=4)
        physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
        cnt, _ = generate_contacts(pairs, max_per_pair=4)
        physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        out = dict(pairs=len(cnt), contacts=int(cnt.sum()))
    else:
        from physx_gb300.solver import joint_frame as gpu_joint_frame
        fr = joint_workload()
        gpu_joint_frame(fr)
        physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
        r = gpu_joint_frame(fr)
        physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        out = dict(joints=len(fr["joint_a"]), headers=len(r["header_start"]))
    print(json.dumps(dict(profiled=which, **{k: (int(v) if hasattr(v, "__int__") else v) for k, v in out.items()})))


def dist_setup(n):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != n:
        sys.exit("bench.py: --gpus %d but WORLD_SIZE is %d (launch N > 1 ranks with torch.distributed.run)" % (n, world))
    if n <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    dist.init_process_group("gloo", init_method="env://")
    return rank, world, dist


def rank_scenes(seed, rank, nb_scenes):
    """The scenes of one rank: every rank steps its own independent scene set
    (weak scaling, no data-path collective)."""
    from physx_gb300.workloads import batched_scenes
    return batched_scenes(seed + 1000 * rank, nb_scenes)


def reduce_over_ranks(ms, bodies, dist):
    """Whole-job figures: the slowest rank's time and the bodies of all ranks."""
    if not dist:
        return ms, bodies
    import torch
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    bt = torch.tensor([bodies], dtype=torch.float64)
    dist.all_reduce(bt)
    return float(t.item()), int(bt.item())


def main():
    a = parse()
    import numpy as np
    if a.profile_extra:
        profile_extra(a.profile_extra)
        return
    rank, world, dist = dist_setup(a.gpus)
    from physx_gb300.workloads import batched_scenes
    from physx_gb300.world import DEFAULT_PARAMS
    cores = os.cpu_count() or 1

    if a.impl == "reference":
        if rank != 0:
            return
        # The reference path on the host cores: the oracle restatement of the
        # frame (the reference build does not travel to this machine), on the same
        # workload, pre-rolled on the CPU as the GPU arm pre-rolls on the device,
        # then --steps consecutive persistent steps after --warmup.
        scenes = batched_scenes(a.seed, a.scenes)
        r = cpu_baseline(scenes, DEFAULT_PARAMS, a.cpu_scenes, a.steps, cores, preroll=a.preroll, warmup=a.warmup)
        line = dict(impl="reference", metric=METRIC, value=r["value"], unit=UNIT, n_gpus=a.gpus, steps=a.steps, warmup=a.warmup,
                    ms_per_step=r["ms_per_step"], higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
                    config=dict(workload=WORKLOAD, scenes=a.scenes, sample_scenes=len(cpu_sample(a.scenes, a.cpu_scenes)),
                                preroll_steps=a.preroll, persistent=True, l2="n/a (CPU)"),
                    cpu_baseline=dict(value=r["value"], unit=UNIT, cores=r["cores"], kind="port", sample=r["sample"]),
                    e2e=dict(value=r["value"], unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line))
        return

    import physx_gb300
    physx_gb300.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from physx_gb300.world import World
    scenes = rank_scenes(a.seed, rank, a.scenes)
    w = World(scenes)
    info = w.info()
    bodies = info["bodies"]
    # pre-roll to a contact-rich state, then warm up (builds the graph)
    w.step(a.preroll, graph=True)
    # block-per-scene threshold for this scene-size histogram, timed on a temporary
    # copy of all scenes in their current state (the world's own state does not
    # advance; a smaller sample would not load the GPU like the full set does)
    if a.large_bodies:
        w.set_large_bodies(a.large_bodies)
        tuned_threshold, tuned_ms = a.large_bodies, 0.0
    else:
        tuned_threshold, tuned_ms = w.autotune(steps=6)
    tuning = w.tuning()
    w.step(a.warmup, graph=True)
    w.synchronize()
    if a.profile_step:
        L = physx_gb300.lib()
        physx_gb300.check(L.gbpx_profiler_start(), "gbpx_profiler_start")
        w.step(a.profile_step, graph=False)
        physx_gb300.check(L.gbpx_profiler_stop(), "gbpx_profiler_stop")
        print(json.dumps(dict(profiled_steps=a.profile_step, kernels_per_step=w.info()["kernels_per_step"],
                              large_bodies=w.info()["large_bodies"], **w.stats())))
        return
    state = w.get_bodies()
    if dist:
        dist.barrier()
    clocks = ClockSampler(smi_gpu_id(int(os.environ.get("LOCAL_RANK", "0"))))
    clocks.start()
    ms = w.time_steps(a.steps, graph=True)
    clk = clocks.stop()
    ms, total_bodies = reduce_over_ranks(ms, bodies, dist)
    status = w.status()
    st = w.stats()
    value = total_bodies * a.steps / (ms / 1000.0)

    # end to end through host memory: upload bodies, step, download, every step
    host_in = w.pinned_bodies()
    host_out = w.pinned_bodies()
    host_out[:] = state
    e2e_ms = 0.0
    for _ in range(a.steps):
        host_in[:] = host_out
        e2e_ms += w.step_host(host_in, host_out, 1, graph=True)
    e2e_value = bodies * a.steps / (e2e_ms / 1000.0)

    # plain comparison: the same scenes, one scene per launch
    counts = scenes["body_count"]
    idx = np.linspace(0, len(counts) - 1, min(a.plain_scenes, len(counts))).astype(np.int64)
    plain_ms = 0.0
    plain_bodies = 0
    for i in idx:
        plain_ms += w.time_plain(int(i), 1)
        plain_bodies += int(counts[i])
    plain_value = plain_bodies / (plain_ms / 1000.0)

    # Per-kernel device times (un-captured steps, CUDA events between the launches on
    # the world's stream) and the roofline of the dominant kernel.  Algorithmic
    # (compulsory) HBM bytes per launch, from the step's own counts:
    #   broadphase   48 B per body (pose, type, shape) + 12 B per pair (key, kind queue)
    #   narrowphase  108 B per pair (two poses and shapes, key, slot, count) + 32 B per contact; persistent
    #                mode adds 8 B per pair (previous slot, friction count) and, per pair of a cached kind
    #                (plane-capsule, plane-box, capsule-box, box-box), its 288 B manifold read and written
    #   batching     280 B per body (PxRigidBodyData in, solver body records out) + 12 B per constraint
    #   preparation  32 B per contact in + 2 x 184 B solver bodies per constraint + packed rows written;
    #                persistent mode adds per constraint a 16 B friction header + one 112 B patch read and written
    #   solve        compulsory: packed rows read once (the resident solve keeps them on chip for all
    #                iterations), plus per body 64 B velocities in, 64 B transform and inertia in,
    #                28 B pose in, 52 B PxRigidBodyData fields written back
    st = w.stats()
    stage_ms = w.time_stages(max(3, a.steps // 3))
    kinds = w.kind_counts()
    nbPos, nbVel = DEFAULT_PARAMS["nb_pos"], DEFAULT_PARAMS["nb_vel"]
    np_ms = sum(v for k, v in stage_ms.items() if k.startswith("np "))
    persistent = bool(DEFAULT_PARAMS["persistent"])
    cached_pairs = sum(kinds[k] for k in ("np plane-capsule", "np plane-box", "np capsule-box", "np box-box"))
    stage_bytes = {
        "broadphase": bodies * 48 + st["pairs"] * 12,
        "narrowphase": st["pairs"] * 108 + st["contacts"] * 32 + (st["pairs"] * 8 + cached_pairs * 576 if persistent else 0),
        "batching": bodies * 280 + st["constraints"] * 12,
        "row preparation": st["contacts"] * 32 + st["constraints"] * 368 + st["row_bytes"] + (st["constraints"] * 256 if persistent else 0),
        "solve": st["row_bytes"] + bodies * (64 + 64 + 28 + 52),
    }
    stage_time = {"broadphase": stage_ms["broadphase"], "narrowphase": np_ms, "batching": stage_ms["batching"],
                  "row preparation": stage_ms["row preparation"], "solve": stage_ms["solve"]}
    peak, peak_kind = measured_peak()
    stages = {k: dict(ms=stage_time[k], gbs=stage_bytes[k] / (stage_time[k] / 1000.0) / 1e9, bytes=stage_bytes[k]) for k in stage_time}
    stages["narrowphase"]["kinds"] = {k[3:]: dict(pairs=kinds[k], ms=stage_ms[k]) for k in kinds}
    # the dominant single kernel: the narrowphase is nine kernels (one per pair kind), so
    # it competes kernel by kernel; a narrowphase kernel's bytes are its share of the
    # stage's by pairs
    kernel_ms = {k: v for k, v in stage_time.items() if k != "narrowphase"}
    kernel_ms.update({k: stage_ms[k] for k in kinds})
    dominant = max(kernel_ms, key=kernel_ms.get)
    if dominant in kinds:
        dom_bytes = stage_bytes["narrowphase"] * kinds[dominant] / max(1, st["pairs"])
    else:
        dom_bytes = stage_bytes[dominant]
    achieved = dom_bytes / (kernel_ms[dominant] / 1000.0) / 1e9
    traffic = profiled_traffic(dominant)
    roofline = dict(bound="hbm", kernel=dominant, achieved=achieved, peak=peak, unit="GB/s", frac=achieved / peak,
                    traffic=traffic, peak_source=peak_kind, algorithmic_bytes_per_launch=dom_bytes, launch_ms=kernel_ms[dominant])
    # the whole step's compulsory HBM bytes, per the scope's measurement model: broadphase
    # 36 B per updated box + 28 B per box + 16 B per active pair; narrowphase 108 B per pair
    # + 32 B per contact (+ 576 B per pair of a cached kind); per body 96 B in + 64 B out; per
    # pair with contacts 208 B of friction patches read and written + 32 B per contact in.
    # Rows are built and consumed on chip and do not count.
    statics = info["statics"]
    bytes_step = (36 * bodies + 28 * (bodies + statics) + 16 * st["pairs"] + st["pairs"] * 108 + st["contacts"] * 32 + cached_pairs * 576 +
                  bodies * (96 + 64) + st["constraints"] * 208 + st["contacts"] * 32)
    step_roofline = dict(algorithmic_bytes_per_step=bytes_step, achieved=bytes_step / (ms / a.steps / 1000.0) / 1e9, unit="GB/s",
                         peak=peak, frac=bytes_step / (ms / a.steps / 1000.0) / 1e9 / peak)
    cpu = None
    if rank == 0:
        # the same sample of the world in the state the timed steps started from
        # (spawned processes: no CUDA state is inherited)
        cpu = cpu_baseline(dict(scenes, rigid=state), DEFAULT_PARAMS, a.cpu_scenes, a.cpu_steps, cores, preroll=0, warmup=1)
        cpu.pop("seconds", None)
        cpu.pop("ms_per_step", None)
    if rank != 0:
        return
    w.release()
    serving = None
    if a.serve_seconds > 0:
        from physx_gb300.serve_load import run_poisson
        serving = run_poisson(duration=a.serve_seconds, rate=a.serve_rate, budget_bytes=a.serve_budget_gb * 1e9, seed=a.seed + 1,
                              lanes_per_class=a.serve_lanes)
        serving["workload"] = ("Poisson %.0f req/s of 'advance scene k by n~U{1..8} steps' over a pool of scenes log-uniform [16,4096] "
                               "bodies admitted against a %.0f GB budget, retired after U(500,5000) steps; %.0f s run" %
                               (a.serve_rate, a.serve_budget_gb, a.serve_seconds))
    extras = None
    if a.extras:
        extras = dict(pyramid=bench_pyramid(a.pyramid_steps), broadphase_1m=bench_broadphase(a.bp_frames, a.bp_cpu_frames),
                      large_scene_100k=bench_large_scene(a.large_steps, a.large_cpu_frames), joints=bench_joints(a.joint_frames, 5),
                      convex_core=bench_convex_core(20, 20000), pgs=bench_pgs(20, 3))
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=a.gpus, steps=a.steps, warmup=a.warmup, ms_per_step=ms / a.steps,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
                config=dict(workload=WORKLOAD, scenes=a.scenes, bodies_per_gpu=bodies, preroll_steps=a.preroll, pairs_per_step=st["pairs"],
                            constraints_per_step=st["constraints"], contacts_per_step=st["contacts"], graph=True,
                            autotune=dict(key="scene-size histogram", large_bodies=tuned_threshold,
                                          solve=SOLVE_VARIANTS[getattr(w, "solve_variant", 8)],
                                          prep_blocks_per_sm=tuning["prep_blocks_per_sm"],
                                          narrowphase_blocks_per_sm=tuning["narrowphase_blocks_per_sm"],
                                          resident_stream_levels=tuning["resident_stream"],
                                          sample_ms_per_step=tuned_ms),
                            l2="inputs larger than L2: resident scene state %.0f MB per GPU" % (info["device_bytes"] / 1e6),
                            parallelism="scene-sharded replicas" if a.gpus > 1 else "single GPU"),
                e2e=dict(value=e2e_value, unit=UNIT, h2d_bytes_per_step=bodies * 96, d2h_bytes_per_step=bodies * 96),
                plain_gpu=dict(value=plain_value, unit=UNIT, sample="%d scenes (%d bodies), one scene per launch" % (len(idx), plain_bodies),
                               batched_over_plain=value / plain_value),
                roofline=roofline, stages=stages, step_roofline=step_roofline, cpu_baseline=cpu, clocks=clk, gpu_launches=a.steps * info["kernels_per_step"],
                contacts_per_s=st["contacts"] * a.steps / (ms / 1000.0), pairs_per_s=st["pairs"] * a.steps / (ms / 1000.0),
                status_nonzero_scenes=int((status != 0).sum()), serving=serving, workloads=extras)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
