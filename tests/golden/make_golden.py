"""Writes the golden fixtures tests/golden/*.npz from the CPU oracle.

Run from the repository root: ``python tests/golden/make_golden.py``. The
oracle itself is pinned by the reference's own unit tests and by the
restatements in tests/test_oracle.py; these fixtures freeze its answers on
cases those tests do not spell out, so later changes to either side show up.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import oracle as O  # noqa: E402
from golden_io import replay  # noqa: E402
from vdb_mapping_gb300 import workloads as W  # noqa: E402
from vdb_mapping_gb300.mapping import Config  # noqa: E402


def pcl(xyz):
    xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
    out = np.ones((xyz.shape[0], 4), np.float32)
    out[:, :3] = xyz
    return out


def save(name, res, cfg, scans, origins):
    case = {
        "resolution": np.float64(res),
        "config": np.array([cfg.max_range, float(cfg.fast_mode), cfg.accumulation_period, cfg.prob_hit,
                            cfg.prob_miss, cfg.prob_thres_min, cfg.prob_thres_max], np.float64),
        "scans": np.stack(scans).astype(np.float32),
        "scan_origins": np.asarray(origins, np.float64),
    }
    c = dict(case)
    c["cfg"], c["res"] = cfg, res
    origins_, values, masks = replay(O.OracleMap(res), c)
    case.update(origins=origins_, values=values, masks=masks)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **case)
    print(f"{name}: {len(origins_)} leaves, {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    rng = np.random.default_rng(1234)
    ref = Config(max_range=10, prob_hit=0.9, prob_miss=0.1, prob_thres_min=0.49, prob_thres_max=0.51)
    mix = Config(max_range=3.0, prob_hit=0.7, prob_miss=0.4, prob_thres_min=0.12, prob_thres_max=0.97)

    # 1. Axis points, negative coordinates, a clipped point and repeats (res 0.1).
    pts = pcl([[0, 0, 0.5], [0, 0, -0.5], [0.3, -0.2, 0.1], [0, 0, 0.7], [-0.45, 0.05, 0.35]])
    save("axis_and_clip", 0.1, Config(max_range=0.6, prob_hit=0.9, prob_miss=0.1, prob_thres_min=0.49,
                                      prob_thres_max=0.51), [pts] * 3, [(0, 0, 0)] * 3)

    # 2. DDA tie families from a far origin at 0.02 m.
    res = 0.02
    o = np.array([5000.013, -3000.007, 40.004])
    ov = np.floor(o / res + 0.5)
    dirs = []
    for p in [(1, 1, 0), (1, 3, 0), (2, 6, 0), (3, 5, 0), (1, 3, 5), (5, 5, 5), (2, 2, 1), (1, 1, 2)]:
        for s in (1, 2, 5, 9):
            for sg in [(1, 1, 1), (-1, 1, -1), (1, -1, 1), (-1, -1, -1)]:
                for perm in [(0, 1, 2), (2, 0, 1), (1, 2, 0)]:
                    dirs.append(np.array(p)[list(perm)] * s * np.array(sg))
    ends = (ov[None, :] + np.array(dirs)) * res
    save("dda_ties_far_origin", res, mix, [pcl(ends)], [o])

    # 3. Quantiser boundaries: coordinates at (k - 1/2) * res and float32 neighbours.
    res = 0.05
    base = []
    for k in range(-30, 31, 3):
        w = np.float32((k - 0.5) * res)
        for v in (w, np.nextafter(w, np.float32(1e9)), np.nextafter(w, np.float32(-1e9))):
            base.append([v, np.float32(0.5 * res * (k % 5)), np.float32(-0.3)])
            base.append([np.float32(0.1), v, np.float32(0.2)])
    save("quantiser_boundaries", res, mix, [pcl(base)], [(0.0125, -0.0375, 0.4)])

    # 4. Room scans, 512 random beams each, three scans (dedup, clamp, hysteresis over scans).
    wl = W.get("small")
    scans, origins = [], []
    for k in range(3):
        p, o = wl.scan(k)
        idx = rng.choice(p.shape[0], 512, replace=False)
        scans.append(p[idx])
        origins.append(o)
    save("room_subsample", wl.resolution, Config(max_range=4.0, prob_hit=0.7, prob_miss=0.4,
                                                 prob_thres_min=0.12, prob_thres_max=0.97), scans, origins)

    # 5. Stress rays (far origin, 0.02 m), 96 rays clipped at 2.5 m, NaN/inf mixed in.
    ws = W.get("stress")
    p, o = ws.scan(0)
    sel = p[rng.choice(p.shape[0], 96, replace=False)].copy()
    sel[3, 0] = np.nan
    sel[7, 2] = np.inf
    save("stress_subsample", ws.resolution, Config(max_range=2.5, prob_hit=0.7, prob_miss=0.4,
                                                   prob_thres_min=0.12, prob_thres_max=0.97), [sel, sel], [o, o])

    # 6. Reference configuration, hits and misses fighting over the same voxels.
    pts = []
    for _ in range(200):
        pts.append(rng.uniform([-2, -2, -1], [2, 2, 1]))
    save("hit_miss_mix", 0.25, ref, [pcl(pts), pcl(pts[::-1]), pcl(pts[50:] + pts[:50])], [(0.1, 0.05, 0.0)] * 3)


if __name__ == "__main__":
    main()
