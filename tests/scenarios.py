"""Seeded synthetic inputs shared by the golden-fixture generator and the tests.

Broadphase frames follow the broadphase-stress workload's shape (centres
uniform in a cube, log-normal half-extents, a random fraction of boxes moved
by N(0, sigma) each frame) plus edge cases the reference handles: touching
faces, +0/-0 coordinates, equal min-X keys, static/kinematic/dynamic groups,
shared (compound) group ids, per-object distances, removals and re-creations.
"""
import numpy as np


def filter_group(kind, i):
    """PxGetBroadPhase{Static,Kinematic,Dynamic}FilterGroup (physx/include/PxBroadPhase.h:264-291)."""
    if kind == 0:
        return 0
    return ((i + 1) << 3) | (1 if kind == 1 else 2)


def bp_frames(seed, n, frames, extent=100.0, move_frac=0.1, sigma=0.2, mu=np.log(0.5), s=0.5, edge_cases=True,
              removals=True, distances=True):
    """Yields dicts with created/updated/removed/bounds/groups/distances/capacity per frame."""
    rng = np.random.default_rng(seed)
    cap = n
    centres = rng.uniform(0.0, extent, size=(n, 3)).astype(np.float32)
    half = np.exp(rng.normal(mu, s, size=(n, 3))).astype(np.float32)
    kinds = rng.choice([0, 1, 2], size=n, p=[0.1, 0.1, 0.8])
    ids = np.arange(n)
    if edge_cases:
        # compound actors: pairs of boxes share a dynamic id
        shared = rng.choice(n, size=max(2, n // 50), replace=False)
        ids[shared[1::2]] = ids[shared[0::2]][: len(shared[1::2])]
        kinds[shared] = 2
    groups = np.array([filter_group(k, i) for k, i in zip(kinds, ids)], dtype=np.uint32)
    dist = (rng.uniform(0.0, 0.05, size=n).astype(np.float32) if distances else np.zeros(n, np.float32))
    bounds = np.zeros((cap + 1, 6), np.float32)
    bounds[:n, :3] = centres - half
    bounds[:n, 3:] = centres + half
    if edge_cases and n >= 16:
        # exact touching faces along x, y, z and a -0/+0 pair, equal min-x keys
        bounds[0] = [0.0, 0.0, 0.0, 1.0, 1.0, 1.0]
        bounds[1] = [1.0, 0.0, 0.0, 2.0, 1.0, 1.0]
        bounds[2] = [0.0, 1.0, 0.0, 1.0, 2.0, 1.0]
        bounds[3] = [0.0, 0.0, 1.0, 1.0, 1.0, 2.0]
        bounds[4] = [-1.0, 5.0, 5.0, -0.0, 6.0, 6.0]
        bounds[5] = [0.0, 5.0, 5.0, 1.0, 6.0, 6.0]
        bounds[6] = [10.0, 10.0, 10.0, 11.0, 11.0, 11.0]
        bounds[7] = [10.0, 10.5, 10.5, 12.0, 12.0, 12.0]
        for k in range(8):
            kinds[k] = 2
            groups[k] = filter_group(2, 100000 + k)
        dist[:8] = 0.0
    live = np.ones(n, bool)
    yield dict(created=np.arange(n, dtype=np.uint32), updated=np.zeros(0, np.uint32), removed=np.zeros(0, np.uint32),
               bounds=bounds.copy(), groups=groups.copy(), distances=dist.copy(), capacity=cap)
    for f in range(1, frames):
        alive = np.flatnonzero(live)
        nmove = max(1, int(len(alive) * move_frac))
        moved = rng.choice(alive, size=nmove, replace=False)
        created = np.zeros(0, np.int64)
        removed = np.zeros(0, np.int64)
        if removals and len(alive) > 8:
            rem_pool = np.setdiff1d(alive, moved)
            rem_pool = rem_pool[rem_pool >= 8]
            if len(rem_pool):
                removed = rng.choice(rem_pool, size=max(1, len(alive) // 100), replace=False)
                live[removed] = False
            dead = np.flatnonzero(~live)
            dead = np.setdiff1d(dead, removed)
            if len(dead):
                created = rng.choice(dead, size=max(1, len(dead) // 2), replace=False)
                live[created] = True
        # displace the moved boxes (and some static ones too: the reference lets
        # the user update any object)
        disp = rng.normal(0.0, sigma, size=(len(moved), 3)).astype(np.float32)
        bounds[moved, :3] += disp
        bounds[moved, 3:] += disp
        if len(created):
            c = rng.uniform(0.0, extent, size=(len(created), 3)).astype(np.float32)
            h = np.exp(rng.normal(mu, s, size=(len(created), 3))).astype(np.float32)
            bounds[created, :3] = c - h
            bounds[created, 3:] = c + h
        if edge_cases and f == 1 and n >= 16:
            # move box 1 so it exactly touches box 0 again from the other side
            bounds[1] = [-1.0, 0.0, 0.0, 0.0, 1.0, 1.0]
            moved = np.union1d(moved, [1])
        yield dict(created=np.sort(created).astype(np.uint32), updated=np.sort(moved).astype(np.uint32),
                   removed=np.sort(removed).astype(np.uint32), bounds=bounds.copy(), groups=groups.copy(),
                   distances=dist.copy(), capacity=cap)


def sorted_pairs(a):
    """Canonical form of a pair list: (n, 2) uint32 with id0 < id1, lexicographically sorted."""
    a = np.asarray(a, dtype=np.uint32).reshape(-1, 2)
    if len(a) == 0:
        return a
    a = np.sort(a, axis=1)
    order = np.lexsort((a[:, 1], a[:, 0]))
    return a[order]
