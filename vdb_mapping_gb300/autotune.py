"""Autotuner of the insertion kernels' launch and layout parameters.

The parameters (``vdbg_tuning``: resident DDA warps per SM, rays a DDA warp
takes from the sorted order at a time, runs an apply block merges at a time,
the L1 edges of the sort's length classes, the block-hash load factor) change
speed only, never the map.
``tune`` times candidates on a sample of the caller's own scans, each on a
fresh map (or batch) so the timed inserts see the same map states, and keeps
the fastest by coordinate descent: one parameter at a time, starting from the
library defaults, in a fixed order.
"""
from __future__ import annotations

import statistics

DEFAULT = {"rays_per_take": 32, "apply_chunk_runs": 2048, "length_edges": (2048, 1024, 512), "hash_load": 0.5,
           "dda_warps_per_sm": 16, "sweep_kernel": 0}

CANDIDATES = {
    "rays_per_take": (8, 16, 32),
    "apply_chunk_runs": (1024, 2048, 4096),
    "length_edges": ((512, 256, 128), (1024, 512, 256), (2048, 1024, 512), (2048, 768, 256)),
    "hash_load": (0.25, 0.5),
    "dda_warps_per_sm": (6, 8, 12, 16, 20),
}


def _measure(make, insert, steps, tuning, warmup, repeats):
    """Median device ms per insert over `steps[warmup:]` with `tuning` on a fresh target."""
    target = make()
    try:
        target.setTuning(tuning)
        for k in range(warmup):
            insert(target, steps[k])
        ms = []
        for _ in range(repeats):
            for k in range(warmup, len(steps)):
                insert(target, steps[k])
                ms.append(target.timings()["total_ms"])
        return statistics.median(ms)
    finally:
        target.close()


def tune(make, insert, steps, warmup=1, repeats=1, candidates=None, log=None):
    """Coordinate-descent search. `make()` returns a fresh OccupancyVDBMapping
    or MapBatch, `insert(target, step)` inserts one step, `steps` is the
    sample. Returns (best tuning dict, [(tuning, ms)] of every evaluation)."""
    cand = dict(CANDIDATES)
    if candidates:
        cand.update(candidates)
    best = dict(DEFAULT)
    table = []
    best_ms = _measure(make, insert, steps, best, warmup, repeats)
    table.append((dict(best), best_ms))
    for name in ("dda_warps_per_sm", "length_edges", "rays_per_take", "apply_chunk_runs", "hash_load"):
        for value in cand[name]:
            if value == best[name]:
                continue
            trial = dict(best)
            trial[name] = value
            ms = _measure(make, insert, steps, trial, warmup, repeats)
            table.append((dict(trial), ms))
            if log:
                log(f"{name}={value}: {ms:.3f} ms")
            if ms < best_ms:
                best, best_ms = trial, ms
    return best, table


def tune_map(resolution, config, scans, source="s", **kw):
    """Tuning for one map fed `scans` [(points, origin)]."""
    from .mapping import OccupancyVDBMapping

    capacity = kw.pop("initial_leaf_capacity", 1 << 20)

    def make():
        m = OccupancyVDBMapping(resolution, initial_leaf_capacity=capacity)
        m.setConfig(config)
        m.addInputSource(source, config.max_range, 0)
        return m

    def insert(m, scan):
        m.insertPointCloud(scan[0], scan[1], source)

    return tune(make, insert, scans, **kw)


def tune_batch(resolutions, configs, steps, initial_leaf_capacity=1 << 21, **kw):
    """Tuning for a batch fed `steps`, each [(points, origin)] with one entry per map."""
    from .mapping import MapBatch

    def make():
        b = MapBatch(resolutions, initial_leaf_capacity=initial_leaf_capacity)
        for i, c in enumerate(configs):
            b.setConfig(i, c)
        return b

    def insert(b, step):
        b.insert([p for p, _ in step], [o for _, o in step])

    return tune(make, insert, steps, **kw)
