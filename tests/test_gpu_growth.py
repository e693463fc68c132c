"""Pool growth across a resident map, against the oracle.

Leaf and block slots live in address ranges reserved when a map is created;
growing a pool backs more of the range with device memory and copies nothing
(VDBMapping.hpp:731-792 allocates OpenVDB leaves one at a time and never moves
the tree either). These tests start maps with pools far too small for their
scans, so every kind of growth happens: on the spot when a marking runs out
(then the marking is re-applied), and ahead of need while a call's kernels
run. The maps must stay bit-identical to the oracle's through all of it.
"""
import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def assert_same(a, b, what):
    ao, av, am = a
    bo, bv, bm = b
    assert ao.shape == bo.shape, f"{what}: {ao.shape[0]} leaves vs {bo.shape[0]}"
    assert np.array_equal(ao, bo), f"{what}: leaf sets differ"
    assert np.array_equal(av.view(np.uint32), bv.view(np.uint32)), f"{what}: log-odds differ"
    assert np.array_equal(am, bm), f"{what}: active masks differ"


def test_pools_grow_in_place_across_resident_map(vdbg, oracle):
    w = W.get("small")
    g = vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=2048, initial_block_capacity=8)
    o = oracle.OracleMap(w.resolution)
    for m in (g, o):
        m.setConfig(w.config)
        m.addInputSource("lidar", w.max_range, 0)
    caps = []
    for k in range(w.n_scans):
        pts, org = w.scan(k)
        g.insertPointCloud(pts, org, "lidar")
        o.insertPointCloud(pts, org, "lidar")
        assert_same(g.exportLeaves(), o.exportLeaves(), f"scan {k}")
        caps.append(g.poolInfo())
    first, last = caps[0], caps[-1]
    # The first scan ran out (grown on the spot), later ones were prepared for.
    assert first["grow_sync"] >= 1
    assert last["grow_ahead"] >= 1
    assert last["leaf_capacity"] > 2048 and last["block_capacity"] > 8
    assert last["leaf_backed"] >= last["leaf_capacity"] >= last["leaves"]
    assert last["leaf_reserved"] >= last["leaf_backed"]


def test_growth_ahead_keeps_dense_scans_off_the_slow_path(vdbg, oracle):
    """Ten consecutive dense street scans into one resident map (clamping and
    hysteresis over repeated updates of a large map), starting from a pool of
    a fraction of the first scan's leaves. After the first scan grew the pool
    on the spot, growth happens ahead of need only. The map equals the
    oracle's bit for bit at the end."""
    w = W.get("dense")
    g = vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=1 << 18)
    o = oracle.OracleMap(w.resolution)
    for m in (g, o):
        m.setConfig(w.config)
        m.addInputSource("lidar", w.max_range, 0)
    sync_after_first = None
    for k in range(10):
        pts, org = w.scan(k)
        g.insertPointCloud(pts, org, "lidar")
        o.insertPointCloud(pts, org, "lidar")
        if k == 0:
            sync_after_first = g.poolInfo()["grow_sync"]
    info = g.poolInfo()
    assert info["grow_sync"] == sync_after_first, info
    assert info["grow_ahead"] >= 1, info
    assert_same(g.exportLeaves(), o.exportLeaves(), "after 10 dense scans")
