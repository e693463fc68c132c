"""GPU parity of batched insertion: independent maps (own resolution, own
config, own sensor) sharing one device pool, one scan per map per call. Every
map must equal, bit for bit, the oracle map that received only its scans, and
the same map inserted alone through the single-map path."""
import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W
from vdb_mapping_gb300.mapping import Config

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def small_batch(n_maps=6, seed=41, n_max=12000):
    return W.BatchedWorkload(seed=seed, n_maps=n_maps, n_steps=3, n_min=300, n_max=n_max)


def oracle_maps(oracle, wl, steps):
    maps = []
    for i in range(wl.n_maps):
        o = oracle.OracleMap(wl.resolutions[i])
        o.setConfig(wl.configs[i])
        o.addInputSource("s", wl.configs[i].max_range, 0)
        for k in range(steps):
            pts, org = wl.scan(i, k)
            o.insertPointCloud(pts, org, "s")
        maps.append(o)
    return maps


def test_batch_matches_oracle_per_map(vdbg, oracle):
    wl = small_batch()
    b = vdbg.MapBatch(wl.resolutions)
    for i, c in enumerate(wl.configs):
        b.setConfig(i, c)
    for k in range(3):
        scans = wl.step(k)
        st = b.insert([p for p, _ in scans], [o for _, o in scans])
        assert st["rays"] > 0
    for i, o in enumerate(oracle_maps(oracle, wl, 3)):
        assert b.leafCount(i) == o.leafCount()
        assert_same_map(b.exportLeaves(i), o.exportLeaves(), f"map {i}")


def test_batch_map_equals_map_inserted_alone(vdbg):
    wl = small_batch(n_maps=4, seed=43)
    b = vdbg.MapBatch(wl.resolutions)
    alone = []
    for i, c in enumerate(wl.configs):
        b.setConfig(i, c)
        g = vdbg.OccupancyVDBMapping(wl.resolutions[i])
        g.setConfig(c)
        g.addInputSource("s", c.max_range, 0)
        alone.append(g)
    for k in range(2):
        scans = wl.step(k)
        b.insert([p for p, _ in scans], [o for _, o in scans])
        for i, (p, o) in enumerate(scans):
            alone[i].insertPointCloud(p, o, "s")
    for i, g in enumerate(alone):
        assert_same_map(b.exportLeaves(i), g.exportLeaves(), f"map {i}")


def test_batch_skipped_maps_and_growth(vdbg, oracle):
    # Tiny pools force leaf- and block-pool growth inside a batched call; a map
    # without points, one with a NaN origin and one with max_range 0 are skipped.
    wl = small_batch(n_maps=5, seed=47, n_max=20000)
    b = vdbg.MapBatch(wl.resolutions, initial_leaf_capacity=64, initial_block_capacity=2)
    cfgs = list(wl.configs)
    cfgs[3] = Config(**{**cfgs[3].__dict__, "max_range": 0.0})
    for i, c in enumerate(cfgs):
        b.setConfig(i, c)
    scans = wl.step(0)
    clouds = [p for p, _ in scans]
    origins = [o for _, o in scans]
    clouds[1] = None
    origins[2] = np.array([np.nan, 0.0, 0.0])
    b.insert(clouds, origins)
    for i in (1, 2, 3):
        assert b.leafCount(i) == 0
    for i in (0, 4):
        o = oracle.OracleMap(wl.resolutions[i])
        o.setConfig(cfgs[i])
        o.addInputSource("s", cfgs[i].max_range, 0)
        o.insertPointCloud(*scans[i], "s")
        assert_same_map(b.exportLeaves(i), o.exportLeaves(), f"map {i}")
    assert b.timings()["retries"] >= 0


def test_batch_argument_errors(vdbg):
    from vdb_mapping_gb300 import VdbgError

    b = vdbg.MapBatch([0.1, 0.2])
    pts = np.array([[0, 0, 1, 1]], np.float32)
    # map 1 has points but no config
    b.setConfig(0, W.default_config(10.0))
    with pytest.raises(VdbgError) as e:
        b.insert([pts, pts], [(0, 0, 0), (0, 0, 0)])
    assert "NOT_CONFIGURED" in str(e.value)
    with pytest.raises(VdbgError):
        b.setConfig(2, W.default_config(10.0))
    # the single-map entry points reject a batch handle
    import ctypes as C

    from vdb_mapping_gb300 import _lib

    lib = vdbg.load()
    cfg = _lib.vdbg_config()
    cfg.max_range, cfg.prob_hit, cfg.prob_miss = 10.0, 0.7, 0.4
    assert lib.vdbg_set_config(b._h, C.byref(cfg)) == _lib.STATUS_CODE["VDBG_ERR_INVALID_ARGUMENT"]
    # a voxel index out of range in one scan (its origin, or an endpoint within
    # max_range): nothing of the batch is marked
    b.setConfig(1, W.default_config(1e7))
    for far_pts, far_origin in ((pts, (1e6, 0, 0)), (np.array([[1e6, 0, 0, 1]], np.float32), (0, 0, 0))):
        with pytest.raises(VdbgError) as e:
            b.insert([pts, far_pts], [(0, 0, 0), far_origin])
        assert "COORD_RANGE" in str(e.value)
        assert b.leafCount(0) == 0 and b.leafCount(1) == 0
    b.setConfig(1, W.default_config(10.0))
    b.insert([pts, pts], [(0, 0, 0), (0, 0, 0)])
    assert b.leafCount(0) == 2 and b.leafCount(1) == 1  # z voxels 0..10 at 0.1 m, 0..5 at 0.2 m
