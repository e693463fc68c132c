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
        # Inputs beyond the stated maximum are refused with their own status.
        big = np.zeros((_lib.VDBG_NOALLOC_MAX_POINTS + 1, 4), np.float32)
        o = (C.c_double * 3)(0.0, 0.0, 0.0)
        s = lib.vdbg_insert_point_cloud_noalloc(fixed, C.c_void_p(big.ctypes.data), big.shape[0], 16, o,
                                                b"lidar", 0, None, None)
        assert s == _lib.STATUS_CODE["VDBG_ERR_SIZE_LIMIT"]
    finally:
        lib.vdbg_destroy(regular)
        lib.vdbg_destroy(fixed)
