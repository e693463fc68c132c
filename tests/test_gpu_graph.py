"""GPU tests of the captured batched step (vdbg_batch_use_graph): the same
scans inserted with graph replay on and off must give bit-identical maps,
through pool growth (the step falls back to separate launches), device-side
inputs at changing addresses (recapture) and a scan out of the index range
(nothing applied)."""
import numpy as np
import pytest

from vdb_mapping_gb300 import VdbgError
from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def make_pair(vdbg, wl, **kw):
    pair = []
    for graph in (True, False):
        b = vdbg.MapBatch(wl.resolutions, **kw)
        for i, c in enumerate(wl.configs):
            b.setConfig(i, c)
        b.useGraph(graph)
        pair.append(b)
    return pair


def assert_pair_equal(pair, n_maps):
    g, p = pair
    for i in range(n_maps):
        assert g.leafCount(i) == p.leafCount(i)
        assert_same_map(g.exportLeaves(i), p.exportLeaves(i), f"map {i}")


def test_graph_equals_launch_loop_over_steps(vdbg):
    wl = W.BatchedWorkload(seed=61, n_maps=6, n_steps=5, n_min=500, n_max=30000)
    pair = make_pair(vdbg, wl, initial_leaf_capacity=1 << 16)
    for k in range(5):
        scans = wl.step(k)
        stats = [b.insert([p for p, _ in scans], [o for _, o in scans]) for b in pair]
        for key in ("rays", "visits", "hits", "updates"):
            assert stats[0][key] == stats[1][key], (k, key)
    assert_pair_equal(pair, wl.n_maps)
    gs = pair[0].graphStats()
    assert gs["replays"] == 5
    assert 1 <= gs["captures"] <= 5
    assert pair[1].graphStats()["replays"] == 0


def test_graph_with_pool_growth(vdbg, oracle):
    # Tiny pools: the captured pass runs out of leaves, the call grows the
    # pools and finishes the step with separate launches, the next step
    # recaptures for the new layout.
    wl = W.BatchedWorkload(seed=63, n_maps=4, n_steps=3, n_min=2000, n_max=20000)
    pair = make_pair(vdbg, wl, initial_leaf_capacity=64, initial_block_capacity=2)
    for k in range(3):
        scans = wl.step(k)
        for b in pair:
            b.insert([p for p, _ in scans], [o for _, o in scans])
    assert_pair_equal(pair, wl.n_maps)
    assert pair[0].graphStats()["captures"] >= 2
    for i in range(wl.n_maps):
        o = oracle.OracleMap(wl.resolutions[i])
        o.setConfig(wl.configs[i])
        o.addInputSource("s", wl.configs[i].max_range, 0)
        for k in range(3):
            o.insertPointCloud(*wl.scan(i, k), "s")
        assert_same_map(pair[0].exportLeaves(i), o.exportLeaves(), f"map {i}")


def test_graph_device_inputs_at_new_addresses(vdbg):
    torch = pytest.importorskip("torch")
    wl = W.BatchedWorkload(seed=65, n_maps=3, n_steps=3, n_min=1000, n_max=8000)
    # Pools large enough that no extension (which changes the kernels'
    # parameters and so updates the graph) happens during the test.
    pair = make_pair(vdbg, wl, initial_leaf_capacity=1 << 20, initial_block_capacity=1 << 14)
    keep = []
    for k in (0, 1, 2, 1, 0):
        scans = wl.step(k)
        pts = np.concatenate([np.concatenate([p[:, :3], np.zeros((len(p), 1), np.float32)], 1) for p, _ in scans])
        counts = [len(p) for p, _ in scans]
        keep.append(torch.from_numpy(pts).cuda())  # every step at a new address
        torch.cuda.synchronize()
        if k == 1 and len(keep) == 4:
            before = pair[0].graphStats()["captures"]
        for b in pair:
            b.insert_packed(keep[-1], counts, [o for _, o in scans])
    assert_pair_equal(pair, wl.n_maps)
    gs = pair[0].graphStats()
    assert gs["replays"] == 5
    info = pair[0].poolInfo()
    assert info["grow_ahead"] == 0 and info["grow_sync"] == 0, info
    assert gs["captures"] == before  # new input addresses replay the same graph


def test_graph_coord_range_leaves_maps_unchanged(vdbg):
    wl = W.BatchedWorkload(seed=67, n_maps=3, n_steps=2, n_min=1000, n_max=4000)
    pair = make_pair(vdbg, wl)
    scans = wl.step(0)
    for b in pair:
        b.insert([p for p, _ in scans], [o for _, o in scans])
    before = [pair[0].exportLeaves(i) for i in range(wl.n_maps)]
    bad = [p.copy() for p, _ in wl.step(1)]
    bad[1][0, :3] = (1e9, 0.0, 0.0)  # an endpoint outside the voxel index range
    for b in pair:
        b.setConfig(1, W.default_config(1e10))
        with pytest.raises(VdbgError) as e:
            b.insert(bad, [o for _, o in wl.step(1)])
        assert "COORD_RANGE" in str(e.value)
        b.setConfig(1, wl.configs[1])
    for i in range(wl.n_maps):
        assert_same_map(pair[0].exportLeaves(i), before[i], f"map {i}")
    scans = wl.step(1)
    for b in pair:
        b.insert([p for p, _ in scans], [o for _, o in scans])
    assert_pair_equal(pair, wl.n_maps)
