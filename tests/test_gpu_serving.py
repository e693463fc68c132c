"""GPU tests of the serving loop (vdbg_server_*): scans submitted from a
host thread at staggered times are inserted in continuously re-formed
batched steps; every map must come out bit-identical to the same scans
inserted alone, in submission order, through the single-map path."""
import threading
import time

import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def test_serving_results_equal_alone(vdbg):
    wl = W.BatchedWorkload(seed=51, n_maps=5, n_steps=4, n_min=500, n_max=30000)
    scans = {(i, k): wl.scan(i, k) for i in range(wl.n_maps) for k in range(4)}
    batch = vdbg.MapBatch(wl.resolutions)
    for i, c in enumerate(wl.configs):
        batch.setConfig(i, c)
    server = vdbg.MapServer(batch)
    order = [(i, k) for k in range(4) for i in range(wl.n_maps)]
    rng = np.random.default_rng(5)

    def producer():
        for j, (i, k) in enumerate(order):
            pts, org = scans[(i, k)]
            while server.submit(i, pts, org, tag=j) != 0:
                time.sleep(0.001)
            time.sleep(float(rng.uniform(0, 0.004)))

    th = threading.Thread(target=producer)
    th.start()
    results = []
    while len(results) < len(order):
        results += server.poll(64, wait_ms=200)
    th.join()
    server.drain()
    st = server.stats()
    server.close()
    assert all(r["status"] == 0 for r in results)
    assert sorted(r["tag"] for r in results) == list(range(len(order)))
    for r in results:
        assert r["submit_ns"] <= r["start_ns"] <= r["done_ns"]
        assert 1 <= r["batch_maps"] <= wl.n_maps
    # per map, completions follow submission order
    for i in range(wl.n_maps):
        tags = [r["tag"] for r in sorted(results, key=lambda r: r["done_ns"]) if r["map"] == i]
        assert tags == sorted(tags)
    assert st["requests_done"] == len(order) and st["steps"] <= len(order)
    for i in range(wl.n_maps):
        g = vdbg.OccupancyVDBMapping(wl.resolutions[i])
        g.setConfig(wl.configs[i])
        g.addInputSource("s", wl.configs[i].max_range, 0)
        for k in range(4):
            g.insertPointCloud(*scans[(i, k)], "s")
        assert_same_map(batch.exportLeaves(i), g.exportLeaves(), f"map {i}")


def test_serving_memory_admission(vdbg):
    # A budget too small for the pool to grow: scans are completed with
    # OUT_OF_MEMORY by admission or by the bounded growth, never beyond it.
    wl = W.BatchedWorkload(seed=53, n_maps=3, n_steps=1, n_min=20000, n_max=40000)
    batch = vdbg.MapBatch(wl.resolutions, initial_leaf_capacity=256)
    for i, c in enumerate(wl.configs):
        batch.setConfig(i, c)
    tiny = np.array([[0.0, 0.0, 0.5, 1.0]], np.float32)
    batch.insert([tiny, None, None], [(0, 0, 0), (0, 0, 0), (0, 0, 0)])  # scratch and run buffers exist
    budget = batch.deviceBytes() + (1 << 20)
    server = vdbg.MapServer(batch, memory_budget_bytes=budget)
    for i in range(wl.n_maps):
        pts, org = wl.scan(i, 0)
        assert server.submit(i, pts, org, tag=i) == 0
    server.drain()
    results = server.poll(16)
    st = server.stats()
    server.close()
    assert len(results) == wl.n_maps
    assert any(r["status"] == 7 for r in results)  # VDBG_ERR_OUT_OF_MEMORY
    assert st["device_bytes"] <= budget
    # the batch stays usable: a scan that fits goes in
    before = batch.leafCount(0)
    batch.insert([tiny, None, None], [(0.05, 0, 0), (0, 0, 0), (0, 0, 0)])
    assert batch.leafCount(0) >= max(before, 1)


def test_serving_queue_backpressure(vdbg):
    wl = W.BatchedWorkload(seed=55, n_maps=2, n_steps=1, n_min=1000, n_max=2000)
    batch = vdbg.MapBatch(wl.resolutions)
    for i, c in enumerate(wl.configs):
        batch.setConfig(i, c)
    server = vdbg.MapServer(batch, queue_capacity=2)
    pts, org = wl.scan(0, 0)
    codes = [server.submit(0, pts, org, tag=j) for j in range(50)]
    assert 13 in codes  # VDBG_ERR_BUSY once two scans are queued
    server.drain()
    done = server.poll(64)
    assert len(done) == codes.count(0)
    server.close()


def test_serving_pipelined_steps_equal_alone(vdbg):
    """Scans queued faster than the device drains them: while one step is
    marked and swept, the next is formed and its upload and ray preparation
    run on the second stream (overlapped_steps counts those steps). Every map
    still equals the same scans inserted alone, in order."""
    wl = W.BatchedWorkload(seed=57, n_maps=4, n_steps=6, n_min=20000, n_max=120000)
    scans = {(i, k): wl.scan(i, k) for i in range(wl.n_maps) for k in range(6)}
    batch = vdbg.MapBatch(wl.resolutions)
    for i, c in enumerate(wl.configs):
        batch.setConfig(i, c)
    server = vdbg.MapServer(batch)
    j = 0
    for k in range(6):
        for i in range(wl.n_maps):
            pts, org = scans[(i, k)]
            assert server.submit(i, pts, org, tag=j) == 0
            j += 1
    server.drain()
    results = server.poll(256)
    st = server.stats()
    server.close()
    assert len(results) == j and all(r["status"] == 0 for r in results)
    assert st["overlapped_steps"] >= 1, st
    for i in range(wl.n_maps):
        g = vdbg.OccupancyVDBMapping(wl.resolutions[i])
        g.setConfig(wl.configs[i])
        g.addInputSource("s", wl.configs[i].max_range, 0)
        for k in range(6):
            g.insertPointCloud(*scans[(i, k)], "s")
        assert_same_map(batch.exportLeaves(i), g.exportLeaves(), f"map {i}")
