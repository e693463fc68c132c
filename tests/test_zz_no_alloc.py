"""The no-allocation insertion entry point (vdbg_insert_point_cloud_noalloc).

Some callers cannot allocate device memory while they run: a real-time
mapping loop cannot afford cudaMalloc's unbounded latency and implicit device
synchronisation inside its cycle, and some host applications own every byte
of device memory through their own pool. For them the library offers one
insertion that takes its per-scan scratch from a fixed array inside the
library. This test drives it through the C ABI and checks, on two calls in a
row, that it leaves exactly the map the regular vdbg_insert_point_cloud
leaves (bit for bit: same leaves, same FP32 log-odds, same active masks, same
counters). It sits in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _new_map(lib, _lib, res, cfg, capacity):
    opts = _lib.vdbg_options()
    opts.initial_leaf_capacity = capacity
    h = C.c_void_p()
    assert lib.vdbg_create(res, C.byref(opts), C.byref(h)) == 0
    c = _lib.vdbg_config()
    c.max_range, c.prob_hit, c.prob_miss = cfg.max_range, cfg.prob_hit, cfg.prob_miss
    c.prob_thres_min, c.prob_thres_max = cfg.prob_thres_min, cfg.prob_thres_max
    assert lib.vdbg_set_config(h, C.byref(c)) == 0
    assert lib.vdbg_add_input_source(h, b"lidar", 0.0, 0.0) == 0
    return h


def _export(lib, h):
    n = C.c_int64()
    assert lib.vdbg_leaf_count(h, C.byref(n)) == 0
    cap = n.value
    origins = np.zeros((cap, 3), np.int32)
    values = np.zeros((cap, 512), np.float32)
    masks = np.zeros((cap, 8), np.uint64)
    assert lib.vdbg_export_leaves(h, cap, origins.ctypes.data, values.ctypes.data, masks.ctypes.data,
                                  C.byref(n)) == 0
    return origins[:n.value], values[:n.value], masks[:n.value]


def _device_bytes(lib, h):
    n = C.c_int64()
    assert lib.vdbg_device_bytes(h, C.byref(n)) == 0
    return n.value


def _insert(lib, _lib, h, pts, org, noalloc):
    o = (C.c_double * 3)(*org)
    st = _lib.vdbg_scan_stats()
    fn = lib.vdbg_insert_point_cloud_noalloc if noalloc else lib.vdbg_insert_point_cloud
    return fn(h, C.c_void_p(pts.ctypes.data), pts.shape[0], 16, o, b"lidar", 0, None, C.byref(st)), st


def test_noalloc_insert_matches_regular_insert_twice(vdbg):
    from vdb_mapping_gb300 import _lib
    from vdb_mapping_gb300 import workloads as W

    lib = _lib.load()
    w = W.get("small")
    regular = _new_map(lib, _lib, w.resolution, w.config, 1 << 18)
    fixed = _new_map(lib, _lib, w.resolution, w.config, 1 << 18)
    try:
        for k in range(2):  # two calls in a row reuse (and must reset) the shared scratch
            pts, org = w.scan(k)
            pts = np.ascontiguousarray(pts)
            o = (C.c_double * 3)(*org)
            st_a, st_b = _lib.vdbg_scan_stats(), _lib.vdbg_scan_stats()
            assert lib.vdbg_insert_point_cloud(regular, C.c_void_p(pts.ctypes.data), pts.shape[0], 16, o,
                                               b"lidar", 0, None, C.byref(st_a)) == 0
            assert lib.vdbg_insert_point_cloud_noalloc(fixed, C.c_void_p(pts.ctypes.data), pts.shape[0], 16, o,
                                                       b"lidar", 0, None, C.byref(st_b)) == 0
            for key in ("rays", "visits", "hits", "updates", "new_leaves", "touched_leaves"):
                assert getattr(st_a, key) == getattr(st_b, key), key
            oa, va, ma = _export(lib, regular)
            ob, vb, mb = _export(lib, fixed)
            assert np.array_equal(oa, ob), f"call {k}: leaf sets differ"
            assert np.array_equal(va.view(np.uint32), vb.view(np.uint32)), f"call {k}: log-odds differ"
            assert np.array_equal(ma, mb), f"call {k}: active masks differ"
        # The calls allocated nothing: the map's device bytes did not move.
        before = _device_bytes(lib, fixed)
        pts, org = w.scan(2)
        assert _insert(lib, _lib, fixed, np.ascontiguousarray(pts), org, True)[0] == 0
        assert _device_bytes(lib, fixed) == before
        # Inputs beyond the stated maximum are refused with their own status.
        big = np.zeros((_lib.VDBG_NOALLOC_MAX_POINTS + 1, 4), np.float32)
        o = (C.c_double * 3)(0.0, 0.0, 0.0)
        s = lib.vdbg_insert_point_cloud_noalloc(fixed, C.c_void_p(big.ctypes.data), big.shape[0], 16, o,
                                                b"lidar", 0, None, None)
        assert s == _lib.STATUS_CODE["VDBG_ERR_SIZE_LIMIT"]
    finally:
        lib.vdbg_destroy(regular)
        lib.vdbg_destroy(fixed)


def test_noalloc_full_pool_leaves_map_unchanged(vdbg):
    """A pool too small for the scan: the call reports OUT_OF_MEMORY, grows
    nothing and leaves the map exactly as it was."""
    from vdb_mapping_gb300 import _lib
    from vdb_mapping_gb300 import workloads as W

    lib = _lib.load()
    w = W.get("small")
    h = _new_map(lib, _lib, w.resolution, w.config, 1 << 18)
    try:
        pts, org = w.scan(0)
        assert _insert(lib, _lib, h, np.ascontiguousarray(pts[::8]), org, False)[0] == 0
        before = _export(lib, h)
        bytes_before = _device_bytes(lib, h)
        small = _new_map(lib, _lib, w.resolution, w.config, 64)
        try:
            assert _insert(lib, _lib, small, np.ascontiguousarray(pts[::64]), org, False)[0] == 0
            small_before, small_bytes = _export(lib, small), _device_bytes(lib, small)
            pts1, org1 = w.scan(5)
            s, _ = _insert(lib, _lib, small, np.ascontiguousarray(pts1), org1, True)
            assert s == _lib.STATUS_CODE["VDBG_ERR_OUT_OF_MEMORY"]
            assert _device_bytes(lib, small) == small_bytes
            after = _export(lib, small)
            for x, y in zip(small_before, after):
                assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
            # and the map still works: a regular insert of a scan that fits
            assert _insert(lib, _lib, small, np.ascontiguousarray(pts[::64]), org, False)[0] == 0
        finally:
            lib.vdbg_destroy(small)
        assert _device_bytes(lib, h) == bytes_before
        for x, y in zip(before, _export(lib, h)):
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
    finally:
        lib.vdbg_destroy(h)


def test_noalloc_change_tracking_after_pool_growth(vdbg):
    """Change tracking on a map whose pool a regular insert has grown: the
    change arrays grow with the pool, so the allocation-free call still runs
    (no SIZE_LIMIT) and reports the same change set as the regular call."""
    from vdb_mapping_gb300 import _lib
    from vdb_mapping_gb300 import workloads as W

    lib = _lib.load()
    w = W.get("small")
    maps = [vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=1024) for _ in range(2)]
    for m in maps:
        m.setConfig(w.config)
        m.addInputSource("lidar", w.max_range, 0)
        m.trackChanges(True)
        for k in range(2):  # grows the pool well past 1024 slots, with room ahead
            pts, org = w.scan(k)
            m.insertPointCloud(pts, org, "lidar")
        assert m.poolInfo()["leaf_capacity"] > 1024
    pts, org = w.scan(2)
    pts = np.ascontiguousarray(pts)
    before = maps[1].deviceBytes()
    assert _insert(lib, _lib, maps[0]._h, pts, org, False)[0] == 0
    assert _insert(lib, _lib, maps[1]._h, pts, org, True)[0] == 0
    assert maps[1].deviceBytes() == before
    ca, cb = maps[0].exportChanges(), maps[1].exportChanges()
    for x, y in zip(ca, cb):
        assert np.array_equal(x, y)
    for x, y in zip(maps[0].exportLeaves(), maps[1].exportLeaves()):
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
    for m in maps:
        m.close()


def test_noalloc_dense_scan_at_the_size_limit(vdbg):
    """A 262,144-point street scan (VDBG_NOALLOC_MAX_POINTS) through the
    allocation-free call equals the regular call's map."""
    from vdb_mapping_gb300 import _lib
    from vdb_mapping_gb300 import workloads as W

    lib = _lib.load()
    w = W.get("dense")
    pts, org = w.scan(0)
    pts = np.ascontiguousarray(pts)
    assert pts.shape[0] == _lib.VDBG_NOALLOC_MAX_POINTS
    regular = _new_map(lib, _lib, w.resolution, w.config, 1 << 21)
    fixed = _new_map(lib, _lib, w.resolution, w.config, 1 << 21)
    try:
        bytes_before = _device_bytes(lib, fixed)
        assert _insert(lib, _lib, regular, pts, org, False)[0] == 0
        s, st = _insert(lib, _lib, fixed, pts, org, True)
        assert s == 0
        assert _device_bytes(lib, fixed) == bytes_before
        for x, y in zip(_export(lib, regular), _export(lib, fixed)):
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
    finally:
        lib.vdbg_destroy(regular)
        lib.vdbg_destroy(fixed)
