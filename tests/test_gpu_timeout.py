"""Bounded device waits: a wait that nothing ends gives up at its bound and
the call returns a timeout status, with the map and the context usable.
The wait is made to run out with the test hook vdbg_test_stall_leaf (a leaf
cell left pending, as if its allocating thread never published the slot);
no GPU fault, trap or hang is involved."""
import time

import numpy as np
import pytest

from vdb_mapping_gb300 import VdbgError
from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def fresh(vdbg, wl):
    g = vdbg.OccupancyVDBMapping(wl.resolution)
    g.setConfig(wl.config)
    g.addInputSource("s", wl.max_range, 0)
    return g


def test_a_stalled_leaf_times_out_and_the_map_recovers(vdbg, oracle):
    wl = W.get("small")
    pts, org = wl.scan(0)
    pts = pts[::8]
    g = fresh(vdbg, wl)
    # every ray starts in the sensor's leaf
    v = oracle.world_to_index(wl.resolution, org)
    lx, ly, lz = (c >> 3 for c in v)
    assert g._lib.vdbg_test_stall_leaf(g._h, -1, lx, ly, lz) == 0
    t0 = time.perf_counter()
    with pytest.raises(VdbgError) as e:
        g.insertPointCloud(pts, org, "s")
    waited = time.perf_counter() - t0
    assert "TIMEOUT" in str(e.value)
    assert waited < 60.0
    # the failed call left nothing behind but the stalled cell
    assert g.leafCount() == 0
    # the context is usable: after a reset the map takes the scan as a fresh one
    g.resetMap()
    g.insertPointCloud(pts, org, "s")
    o = oracle.OracleMap(wl.resolution)
    o.setConfig(wl.config)
    o.addInputSource("s", wl.max_range, 0)
    o.insertPointCloud(pts, org, "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "after the timeout and a reset")


def test_stalling_an_existing_leaf_is_refused(vdbg):
    wl = W.get("small")
    pts, org = wl.scan(0)
    g = fresh(vdbg, wl)
    g.insertPointCloud(pts[::8], org, "s")
    o, _, _ = g.exportLeaves()
    lx, ly, lz = (int(c) >> 3 for c in o[0])
    assert g._lib.vdbg_test_stall_leaf(g._h, -1, lx, ly, lz) != 0
