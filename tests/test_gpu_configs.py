"""GPU parity on the benchmark configs at full size, through digests.

Exporting a map of tens of millions of leaves to compare it voxel by voxel is
impractical, so these tests compare exact digests instead (vdbg_ray_digests,
vdbg_map_digest; the oracle computes the same definitions from its own
traversal and map):

* precision stress, all 20 scans of 65,536 rays from (5000,-3000,40) m at
  0.02 m with 1% of the endpoints on voxel faces and DDA tie directions:
  every ray's castRayIntoGrid path (visit count, voxel sequence hash, end
  voxel, clip flag) equals the oracle's FP64 DDA (VDBMapping.hpp:550-566,
  612-631): the voxel mismatch count is 0;
* the same 20 scans, subsampled, inserted into one resident map: the map
  digest (every leaf, every FP32 log-odds bit pattern, every active bit)
  equals the oracle map's;
* batched, the full 32-map configuration for two steps: every map's digest
  equals the oracle map that received only its scans.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_stress_ray_paths_all_scans(vdbg, oracle):
    w = W.get("stress")
    g = vdbg.OccupancyVDBMapping(w.resolution)
    g.setConfig(w.config)
    mismatched, visits = 0, 0
    for k in range(w.n_scans):
        pts, org = w.scan(k)
        dg = g.rayDigests(pts, org, w.max_range)
        do = oracle.ray_digests(pts, org, w.max_range, w.resolution)
        bad = np.any(dg != do, axis=1)
        mismatched += int(bad.sum())
        visits += int((do[:, 0] & ((1 << 40) - 1)).sum())
        assert int((do[:, 0] >> 41).sum()) == pts.shape[0], "every stress ray is valid"
    assert visits > 3_000_000_000 // 2  # long rays: ~1.6G voxel visits over the config
    assert mismatched == 0, f"{mismatched} rays with a different voxel path"


def test_stress_resident_map_digest(vdbg, oracle):
    w = W.get("stress")
    g = vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=1 << 20)
    o = oracle.OracleMap(w.resolution)
    for m in (g, o):
        m.setConfig(w.config)
        m.addInputSource("s", w.max_range, 0)
    for k in range(w.n_scans):
        pts, org = w.scan(k)
        sub = np.ascontiguousarray(pts[k % 64::64])
        g.insertPointCloud(sub, org, "s")
        o.insertPointCloud(sub, org, "s")
        assert g.last_stats["updates"] == o.last_stats["updates"], f"scan {k}"
    dg, do = g.mapDigest(), o.mapDigest()
    assert dg[0] > 1_000_000, dg
    assert dg == do


def test_batched_full_config_matches_oracle_per_map(vdbg, oracle):
    wl = W.get("batched")
    b = vdbg.MapBatch(wl.resolutions, initial_leaf_capacity=1 << 22)
    for i, c in enumerate(wl.configs):
        b.setConfig(i, c)
    steps = [wl.step(k) for k in range(2)]
    for scans in steps:
        b.insert([p for p, _ in scans], [o for _, o in scans])

    def oracle_digest(i):
        o = oracle.OracleMap(wl.resolutions[i])
        o.setConfig(wl.configs[i])
        o.addInputSource("s", wl.configs[i].max_range, 0)
        for scans in steps:
            o.insertPointCloud(*scans[i], "s")
        return o.mapDigest()

    with ThreadPoolExecutor(max_workers=8) as ex:
        expected = list(ex.map(oracle_digest, range(wl.n_maps)))
    for i in range(wl.n_maps):
        assert b.mapDigest(i) == expected[i], f"map {i}"
    assert sum(d[0] for d in expected) > 100_000
