"""GPU parity of the volume ray intersector paths against the oracle:
raytrace queries (VDBMapping.hpp:675-721) and fast-mode insertion
(castRayIntoGridFast, VDBMapping.hpp:577-602). Bit-exact: success flags, end
points as float64 bit patterns, maps and scan statistics."""
import dataclasses

import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map
from test_oracle_raytrace import EMPTY_LO, EMPTY_HI, vdb_bit

pytestmark = pytest.mark.gpu


def same_trace(g, o, what=""):
    gok, gend = g
    r, ook, oend = o
    assert r == 0, what
    assert np.array_equal(gok, ook), (what, np.flatnonzero(gok != ook)[:10])
    assert np.array_equal(gend.view(np.uint64), oend.view(np.uint64)), what


def active_pair(vdbg, oracle, voxels, res=1.0):
    g = vdbg.OccupancyVDBMapping(res)
    o = oracle.OracleMap(res)
    leaves = {}
    for v in voxels:
        key = tuple(c & ~7 for c in v)
        w, b = vdb_bit(*v)
        leaves.setdefault(key, np.zeros(8, np.uint64))[w] |= np.uint64(1) << np.uint64(b)
    origins = np.array(list(leaves.keys()), np.int32).reshape(-1, 3)
    masks = np.array(list(leaves.values()), np.uint64).reshape(-1, 8)
    for m in (g, o):
        m.applyMapSectionStates(EMPTY_LO, EMPTY_HI, origins, masks)
    return g, o


def test_raytrace_known_answers(vdbg, oracle):
    g, o = active_pair(vdbg, oracle, [(10, 0, 0)])
    org = np.array([[0.5, 0.5, 0.5], [0.5, 20.5, 0.5], [10.5, 0.5, 0.5], [20.5, 0.5, 0.5], [0.5, 0.5, 0.5]])
    d = np.array([[1, 0, 0], [1, 0, 0], [1, 0, 0], [-1, 0, 0], [7, 0, 0]], np.float64)
    ln = np.array([20.0, 16.0, 16.0, 16.0, 20.0])
    ok, ends = g.raytrace(org, d, ln)
    assert ok.tolist() == [True, False, True, True, True]
    assert ends.tolist() == [[10, 0, 0], [16.5, 20.5, 0.5], [17, 0, 0], [10, 0, 0], [10, 0, 0]]
    same_trace((ok, ends), o.raytrace(org, d, ln))


def built_pair(vdbg, oracle):
    wl = W.get("small")
    g = vdbg.OccupancyVDBMapping(wl.resolution)
    o = oracle.OracleMap(wl.resolution)
    for m in (g, o):
        m.setConfig(wl.config)
        m.addInputSource("s", wl.max_range, 0)
    for k in (0, 0, 0, 0, 0, 1, 2):  # repeated hits turn voxels active
        pts, org = wl.scan(k)
        g.insertPointCloud(pts[::4], org, "s")
        o.insertPointCloud(pts[::4], org, "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "built maps")
    return wl, g, o


def queries(wl, n, seed):
    rng = np.random.default_rng(seed)
    sensors = np.array([wl.scan(k)[1] for k in range(3)], np.float64)
    org = sensors[np.arange(n) % 3] + rng.normal(0, 0.3, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    d[:, 2] *= 0.2
    d[: n // 8, 1:] = 0.0                            # along x
    d[n // 8: n // 4, 0] = d[n // 8: n // 4, 1]      # |dx| = |dy|
    d[n // 4: n // 4 + 4] = 0.0                      # no direction
    far = slice(n // 2, n // 2 + n // 8)            # from 100 m out, mostly away from the map
    org[far] = org[far] + np.array([100.0, 0.0, 0.0])
    ln = rng.uniform(0.5, 40.0, n)
    return org, d, ln


def n_min(ok):
    return len(ok) // 50


def test_raytrace_matches_oracle_on_a_scanned_map(vdbg, oracle):
    wl, g, o = built_pair(vdbg, oracle)
    org, d, ln = queries(wl, 4096, 5)
    res = g.raytrace(org, d, ln)
    same_trace(res, o.raytrace(org, d, ln), "scanned map")
    ok, _ = res
    assert ok.sum() > n_min(ok) and (~ok).sum() > n_min(ok)  # both outcomes occur


def test_raytrace_of_a_batch_map(vdbg, oracle):
    wl = W.get("small")
    b = vdbg.MapBatch([0.2, wl.resolution])
    b.setConfig(0, W.default_config(5.0))
    b.setConfig(1, wl.config)
    o = oracle.OracleMap(wl.resolution)
    o.setConfig(wl.config)
    o.addInputSource("s", wl.max_range, 0)
    for k in (0, 0, 0, 0, 0, 1):
        pts, org = wl.scan(k)
        b.insert([pts[::16], pts[::4]], [org, org])
        o.insertPointCloud(pts[::4], org, "s")
    org, d, ln = queries(wl, 1024, 7)
    same_trace(b.raytrace(1, org, d, ln), o.raytrace(org, d, ln), "batch map 1")


def test_raytrace_range_error(vdbg):
    from vdb_mapping_gb300 import VdbgError

    g = vdbg.OccupancyVDBMapping(1.0)
    with pytest.raises(VdbgError):
        g.raytrace([[2e9, 0, 0]], [[1, 0, 0]], 1.0)


def fast_config(wl):
    return dataclasses.replace(wl.config, fast_mode=True)


def test_fast_mode_matches_oracle(vdbg, oracle):
    wl, g, o = built_pair(vdbg, oracle)
    cfg = fast_config(wl)
    g.setConfig(cfg)
    o.setConfig(cfg)
    for k in (3, 4, 5, 1):
        pts, org = wl.scan(k)
        g.insertPointCloud(pts[::2], org, "s")
        o.insertPointCloud(pts[::2], org, "s")
        sg = g.last_stats
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"fast scan {k}")
        for key in ("rays", "visits", "hits"):
            assert sg[key] == o.last_stats[key], (k, key, sg[key], o.last_stats[key])


def test_raytrace_and_fast_mode_share_span_buffers(vdbg, oracle):
    """Fast mode and raytrace keep their span records in the same device
    buffers: fast inserts, raytraces that grow the query buffer and the span
    buffers, then fast inserts again, all equal to the oracle."""
    wl, g, o = built_pair(vdbg, oracle)
    cfg = fast_config(wl)
    g.setConfig(cfg)
    o.setConfig(cfg)
    step = 0
    for n in (256, 16384, 65536):
        pts, org = wl.scan(3 + step % 3)
        g.insertPointCloud(pts[::8], org, "s")
        o.insertPointCloud(pts[::8], org, "s")
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"fast insert before {n} queries")
        q_org, d, ln = queries(wl, n, 11 + step)
        same_trace(g.raytrace(q_org, d, ln), o.raytrace(q_org, d, ln), f"{n} queries")
        step += 1
    pts, org = wl.scan(1)
    g.insertPointCloud(pts, org, "s")
    o.insertPointCloud(pts, org, "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "fast insert after the queries")


def test_fast_mode_from_an_empty_map(vdbg, oracle):
    wl = W.get("small")
    cfg = fast_config(wl)
    g = vdbg.OccupancyVDBMapping(wl.resolution)
    o = oracle.OracleMap(wl.resolution)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource("s", wl.max_range, 0)
    marked = 0
    for k in (0, 0, 0, 0, 0, 0, 1, 2):  # the sixth hit turns voxels active; then they take misses
        pts, org = wl.scan(k)
        g.insertPointCloud(pts[::4], org, "s")
        o.insertPointCloud(pts[::4], org, "s")
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"fast from empty, scan {k}")
        assert g.last_stats["visits"] == o.last_stats["visits"]
        marked += o.last_stats["visits"] - o.last_stats["hits"]
    assert marked > 0


def test_fast_mode_rejected_where_unsupported(vdbg):
    from vdb_mapping_gb300 import VdbgError

    wl = W.get("small")
    b = vdbg.MapBatch([wl.resolution, wl.resolution])
    with pytest.raises(VdbgError):
        b.setConfig(0, fast_config(wl))
