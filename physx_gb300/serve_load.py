"""Open-loop serving load: Poisson arrivals of "advance scene k by n steps"
requests over a live pool of resident scenes (seeded, synthetic).

Scenes have body counts log-uniform in [nmin, nmax] (sphere / box / capsule
dropped onto a plane, as the batched workload); each is retired after a
lifetime of U(life) steps once it owes no steps, and a new scene takes its
place.  Latency of a request runs from its scheduled arrival time to the
server observing its last step done (server clock), so loop lag counts.  The
load loop itself runs in the library (gbpx_server_run_load).
"""
import numpy as np

from .server import Server, slots_for_budget
from .workloads import batched_scenes

CLASSES = (16, 32, 64, 128, 256, 512, 1024, 2048, 4096)


def scene_library(seed, per_class, nmin, nmax, classes=CLASSES):
    """Pre-generated scenes per capacity class (admitted repeatedly as new scenes)."""
    rng = np.random.default_rng(seed)
    lib = {c: [] for c in classes}
    lo = [nmin] + [c + 1 for c in classes[:-1]]
    for c, l in zip(classes, lo):
        if c < nmin or l > nmax:
            continue
        for k in range(per_class):
            a, b = max(l, nmin), min(c, nmax)
            n = int(np.clip(np.exp(rng.uniform(np.log(a), np.log(b + 1))), a, b))
            sc = batched_scenes(int(rng.integers(1 << 30)), 1, nmin=n, nmax=n)
            lib[c].append(dict(rigid=sc["rigid"], types=sc["types"], geoms=sc["geoms"], friction=sc["friction"],
                               static_poses=sc["static_poses"], static_types=sc["static_types"], static_geoms=sc["static_geoms"]))
    return lib


def run_poisson(duration=10.0, rate=20000.0, budget_bytes=150e9, nmin=16, nmax=4096, steps=(1, 8), life=(500, 5000), seed=5,
                per_class=8, max_scenes=None, lanes_per_class=1):
    """Runs the load for `duration` seconds in the library (gbpx_server_run_load: the
    arrivals, pump, completions, retirements and re-admissions all run natively) and
    returns a summary dict."""
    classes = [c for c in CLASSES if c >= nmin and c // 2 < nmax]
    slots = slots_for_budget(classes, budget_bytes)
    if max_scenes:
        slots = [max(1, min(s, max_scenes // len(classes))) for s in slots]
    lib = scene_library(seed + 1, per_class, nmin, nmax, classes)
    library = [sc for c in classes for sc in lib[c]]   # class picked uniformly, then a scene: log-uniform body counts
    srv = Server(classes, slots, lanes_per_class=lanes_per_class)
    r = srv.run_load(library, duration, rate, steps=steps, life=life, seed=seed)
    srv.release()
    el = r["seconds"]
    return dict(duration_s=el, rate_per_s=rate, submitted=int(r["submitted"]), completed=int(r["completed"]),
                completed_per_s=r["completed"] / el, body_steps_per_s=r["body_steps"] / el, p50_ms=r["p50_ms"], p99_ms=r["p99_ms"],
                p50_ms_512=r["p50_ms_512"], p99_ms_512=r["p99_ms_512"], p50_ms_per_step_512=r["p50_ms_per_step_512"],
                p99_ms_per_step_512=r["p99_ms_per_step_512"], live_scenes=int(r["live_scenes"]), pool_slots=int(sum(slots)),
                retired=int(r["retired"]), admitted_after_start=int(r["admitted_after_start"]), lane_steps=int(r["lane_steps"]),
                lanes=int(r["lanes"]), lanes_per_class=lanes_per_class, classes=list(classes), slots=[int(s) for s in slots])
