"""Open-loop serving load: Poisson arrivals of "advance scene k by n steps"
requests over a live pool of resident scenes (seeded, synthetic).

Scenes have body counts log-uniform in [nmin, nmax] (sphere / box / capsule
dropped onto a plane, as the batched workload); each is retired after a
lifetime of U(life) steps once it owes no steps, and a new scene takes its
place.  Latency of a request runs from its scheduled arrival time to the
server observing its last step done (server clock), so client lag counts.
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
                per_class=8, max_scenes=None):
    """Runs the load for `duration` seconds and returns a summary dict."""
    rng = np.random.default_rng(seed)
    classes = [c for c in CLASSES if c >= nmin and c // 2 < nmax]
    slots = slots_for_budget(classes, budget_bytes)
    if max_scenes:
        slots = [max(1, min(s, max_scenes // len(classes))) for s in slots]
    lib = scene_library(seed + 1, per_class, nmin, nmax, classes)
    srv = Server(classes, slots)
    live, sizes, lifetime, owed, done_steps = [], {}, {}, {}, {}

    def admit_one():
        # body count log-uniform: pick the class by octave, a library scene within it
        c = classes[int(rng.integers(len(classes)))]
        sc = lib[c][int(rng.integers(len(lib[c])))]
        try:
            sid = srv.admit(sc)
        except Exception:
            return False
        live.append(sid)
        sizes[sid] = len(sc["rigid"])
        lifetime[sid] = int(rng.integers(life[0], life[1] + 1))
        owed[sid] = 0
        done_steps[sid] = 0
        return True

    fails = 0
    while fails < 50:
        fails = 0 if admit_one() else fails + 1
    req_scene, req_steps, lat_all, lat_scene, lat_steps = {}, {}, [], [], []
    tag = 0
    t0 = srv.clock()
    t_next = t0
    t_end = t0 + duration
    retired = admitted = 0
    while True:
        now = srv.clock()
        if now >= t_end:
            break
        while t_next <= now:
            sid = live[int(rng.integers(len(live)))]
            n = int(rng.integers(steps[0], steps[1] + 1))
            srv.submit(sid, n, tag, t_next)
            req_scene[tag], req_steps[tag] = sid, n
            owed[sid] += n
            tag += 1
            t_next += rng.exponential(1.0 / rate)
        srv.pump()
        tags, lats = srv.poll()
        for t, l_ in zip(tags.tolist(), lats.tolist()):
            sid = req_scene.pop(t)
            n = req_steps.pop(t)
            owed[sid] -= n
            done_steps[sid] += n
            lat_all.append(l_)
            lat_scene.append(sizes[sid])
            lat_steps.append(n)
            if owed[sid] == 0 and done_steps[sid] >= lifetime[sid] and len(live) > 1:
                srv.retire(sid)
                live.remove(sid)
                retired += 1
                admitted += 1 if admit_one() else 0
    elapsed = srv.clock() - t0
    st = srv.stats()
    srv.release()
    lat = np.array(lat_all)
    sz = np.array(lat_scene)
    m512 = (sz > 256) & (sz <= 512)
    per_step = lat / np.maximum(np.array(lat_steps), 1)   # a request of n steps: its latency per step
    pct = lambda a, q: float(np.percentile(a, q) * 1000.0) if len(a) else None  # noqa: E731
    return dict(duration_s=elapsed, rate_per_s=rate, submitted=tag, completed=len(lat), completed_per_s=len(lat) / elapsed,
                body_steps_per_s=st["body_steps"] / elapsed, p50_ms=pct(lat, 50), p99_ms=pct(lat, 99), p50_ms_512=pct(lat[m512], 50),
                p99_ms_512=pct(lat[m512], 99), p50_ms_per_step_512=pct(per_step[m512], 50), p99_ms_per_step_512=pct(per_step[m512], 99),
                live_scenes=st["live"], pool_slots=int(sum(slots)), retired=retired,
                admitted_after_start=admitted, classes=list(classes), slots=[int(s) for s in slots])
