"""The change set (updateMap's change grid, VDBMapping.hpp:733-781) against
the oracle's, scan by scan: the voxels whose active state flipped, and among
them the ones a hit turned on."""
import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W
from vdb_mapping_gb300.mapping import Config

pytestmark = pytest.mark.gpu

FLIPPY = dict(prob_hit=0.9, prob_miss=0.1, prob_thres_max=0.51, prob_thres_min=0.49)


def same_changes(a, b, what):
    for x, y, name in zip(a, b, ("origins", "active", "value")):
        assert x.shape == y.shape, f"{what}: {name} shape {x.shape} vs {y.shape}"
        assert np.array_equal(x, y), f"{what}: {name} differ"


def test_change_sets_match_oracle(vdbg, oracle):
    w = W.get("small")
    cfg = Config(max_range=w.max_range, **FLIPPY)
    g = vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=4096)
    g.trackChanges(True)
    o = oracle.OracleMap(w.resolution)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource("s", w.max_range, 0)
    flips = 0
    for k in range(4):
        pts, org = w.scan(k)
        g.insertPointCloud(pts, org, "s")
        o.insertPointCloud(pts, org, "s")
        gc, oc = g.exportChanges(), o.exportChanges()
        same_changes(gc, oc, f"scan {k}")
        flips += int(sum(bin(int(v)).count("1") for v in gc[1].ravel()))
    assert flips > 10000


def test_change_set_of_update_map_and_empty_calls(vdbg, oracle):
    w = W.get("small")
    cfg = Config(max_range=w.max_range, **FLIPPY)
    g = vdbg.OccupancyVDBMapping(w.resolution)
    g.trackChanges(True)
    o = oracle.OracleMap(w.resolution)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource("a", w.max_range, 0)
    pts, org = w.scan(0)
    g.raycastPointCloud(pts, org, w.max_range, "a")
    g.updateMap("a")
    o.insertPointCloud(pts, org, "a")
    same_changes(g.exportChanges(), o.exportChanges(), "updateMap")
    # a call that integrates nothing leaves an empty change set
    g.insertPointCloud(np.zeros((0, 4), np.float32), org, "a")
    assert g.exportChanges()[0].shape[0] == 0
    g.trackChanges(False)
    from vdb_mapping_gb300 import VdbgError

    with pytest.raises(VdbgError):
        g.exportChanges()


def test_batch_change_sets_per_map(vdbg, oracle):
    wl = W.BatchedWorkload(seed=71, n_maps=3, n_steps=2, n_min=2000, n_max=9000)
    cfgs = [Config(max_range=c.max_range, **FLIPPY) for c in wl.configs]
    b = vdbg.MapBatch(wl.resolutions)
    b.trackChanges(True)
    ors = []
    for i, c in enumerate(cfgs):
        b.setConfig(i, c)
        o = oracle.OracleMap(wl.resolutions[i])
        o.setConfig(c)
        o.addInputSource("s", c.max_range, 0)
        ors.append(o)
    for k in range(2):
        st = wl.step(k)
        b.insert([p for p, _ in st], [o for _, o in st])
        for i, (p, org) in enumerate(st):
            ors[i].insertPointCloud(p, org, "s")
            same_changes(b.exportChanges(i), ors[i].exportChanges(), f"step {k} map {i}")
