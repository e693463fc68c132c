"""Known answers for the oracle's restatement of the volume ray intersector
paths: raytrace (VDBMapping.hpp:675-721) and fast mode (castRayIntoGridFast,
VDBMapping.hpp:577-602). The reference has no tests for either; the answers
are derived by hand from OpenVDB's published ray, DDA and hierarchical DDA
rules as the oracle states them (1 m voxels, so index = world)."""
import numpy as np

from vdb_mapping_gb300 import workloads as W

EMPTY_LO, EMPTY_HI = (1, 1, 1), (0, 0, 0)  # an empty box: applyMapSectionStates clears nothing


def vdb_bit(x, y, z):
    """(word, bit) of voxel (x, y, z) in OpenVDB's leaf order."""
    off = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7)
    return off >> 6, off & 63


def map_with_active(oracle, voxels, fast=False):
    m = oracle.OracleMap(1.0)
    cfg = W.default_config(100.0)
    cfg.fast_mode = fast
    assert m.setConfig(cfg) == 0
    m.addInputSource("s", 100.0, 0)
    leaves = {}
    for v in voxels:
        o = tuple(c & ~7 for c in v)
        w, b = vdb_bit(*v)
        leaves.setdefault(o, np.zeros(8, np.uint64))[w] |= np.uint64(1) << np.uint64(b)
    origins = np.array(list(leaves.keys()), np.int32).reshape(-1, 3)
    masks = np.array(list(leaves.values()), np.uint64).reshape(-1, 8)
    m.applyMapSectionStates(EMPTY_LO, EMPTY_HI, origins, masks)
    return m


def trace(m, o, d, ln):
    r, ok, ends = m.raytrace([o], [d], ln)
    assert r == 0
    return bool(ok[0]), tuple(ends[0])


def test_raytrace_stops_at_the_first_active_voxel(oracle):
    m = map_with_active(oracle, [(10, 0, 0)])
    assert trace(m, (0.5, 0.5, 0.5), (1, 0, 0), 20.0) == (True, (10.0, 0.0, 0.0))


def test_raytrace_without_an_active_voxel_on_the_span(oracle):
    # The span is leaf (8,0,0), t in [0.46875, 0.96875]; the voxel DDA passes
    # it (voxel 16 enters at exactly t1) and ends one voxel later, still a
    # success.
    m = map_with_active(oracle, [(10, 3, 0)])
    assert trace(m, (0.5, 0.5, 0.5), (1, 0, 0), 16.0) == (True, (17.0, 0.0, 0.0))


def test_raytrace_missing_every_leaf(oracle):
    m = map_with_active(oracle, [(10, 0, 0)])
    assert trace(m, (0.5, 20.5, 0.5), (1, 0, 0), 16.0) == (False, (16.5, 20.5, 0.5))


def test_raytrace_does_not_test_its_start_voxel(oracle):
    m = map_with_active(oracle, [(10, 0, 0)])
    assert trace(m, (10.5, 0.5, 0.5), (1, 0, 0), 16.0) == (True, (17.0, 0.0, 0.0))


def test_raytrace_negative_direction_from_a_leaf_boundary(oracle):
    # The clipped ray starts exactly on x = 16: floor puts the start in the
    # cell being left, whose next crossing is at the same time.
    m = map_with_active(oracle, [(10, 0, 0)])
    assert trace(m, (20.5, 0.5, 0.5), (-1, 0, 0), 16.0) == (True, (10.0, 0.0, 0.0))


def test_raytrace_direction_is_normalised(oracle):
    m = map_with_active(oracle, [(10, 0, 0)])
    assert trace(m, (0.5, 0.5, 0.5), (7.0, 0, 0), 20.0) == trace(m, (0.5, 0.5, 0.5), (1, 0, 0), 20.0)


def test_raytrace_far_query_is_rejected(oracle):
    m = map_with_active(oracle, [(10, 0, 0)])
    r, _, _ = m.raytrace([(2e9, 0, 0)], [(1, 0, 0)], 1.0)
    assert r == 6  # kCoordRange


def test_fast_mode_marks_only_active_voxels(oracle):
    m = map_with_active(oracle, [(5, 0, 0), (6, 0, 0)], fast=True)
    lo = m.logOdds()
    lo_hit, lo_miss = lo["hit"], lo["miss"]
    pts = np.array([[10.2, 0.2, 0.2]], np.float32)
    m.insertPointCloud(pts, (0.2, 0.2, 0.2), "s")
    assert m.last_stats["visits"] == 3 and m.last_stats["hits"] == 1
    for x in range(0, 12):
        want = lo_miss if x in (5, 6) else (lo_hit if x == 10 else 0.0)
        assert m.getValue((x, 0, 0)) == np.float32(want), x
    assert m.isValueOn((5, 0, 0)) and m.isValueOn((6, 0, 0)) and not m.isValueOn((10, 0, 0))
    # the same scan again: the refreshed intersector also holds leaf (8,0,0)
    m.insertPointCloud(pts, (0.2, 0.2, 0.2), "s")
    assert m.getValue((5, 0, 0)) == np.float32(np.float32(lo_miss) + np.float32(lo_miss))
    assert m.getValue((9, 0, 0)) == 0.0


def test_fast_mode_on_an_empty_map_marks_hits_only(oracle):
    m = oracle.OracleMap(1.0)
    cfg = W.default_config(100.0)
    cfg.fast_mode = True
    m.setConfig(cfg)
    m.addInputSource("s", 100.0, 0)
    m.insertPointCloud(np.array([[10.2, 0.2, 0.2]], np.float32), (0.2, 0.2, 0.2), "s")
    assert m.last_stats["visits"] == 1
    o, v, _ = m.exportLeaves()
    assert [tuple(x) for x in o] == [(8, 0, 0)]
    assert np.count_nonzero(v) == 1


def test_normal_mode_marks_the_whole_ray(oracle):
    m = map_with_active(oracle, [(5, 0, 0), (6, 0, 0)], fast=False)
    lo_miss = m.logOdds()["miss"]
    m.insertPointCloud(np.array([[10.2, 0.2, 0.2]], np.float32), (0.2, 0.2, 0.2), "s")
    assert all(m.getValue((x, 0, 0)) == np.float32(lo_miss) for x in range(10))
