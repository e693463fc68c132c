"""GPU parity of artificial areas (VDBMapping.hpp:1152-1236 and the
re-activation in updateMap, :785-789) against the oracle: walls, polygons,
re-activation after non-empty updates only, restoreMapIntegrity. Bit-exact
maps."""
import dataclasses

import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def pair(vdbg, oracle, res, cfg, max_range):
    g = vdbg.OccupancyVDBMapping(res)
    o = oracle.OracleMap(res)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource("s", max_range, 0)
    return g, o


def both(g, o, name, *args):
    getattr(g, name)(*args)
    getattr(o, name)(*args)


def test_wall_reactivation_and_restore_known_answers(vdbg, oracle):
    g, o = pair(vdbg, oracle, 1.0, W.default_config(100.0), 100.0)
    both(g, o, "addArtificialWall", (2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 2.0)
    both(g, o, "integrateUpdate")  # nothing accumulated: no re-activation
    assert len(g.exportLeaves()[0]) == 0
    ray = np.array([[10.0, 5.0, 0.0]], np.float32)
    for _ in range(6):
        both(g, o, "insertPointCloud", ray, (0.0, 5.0, 0.0), "s")
        assert_same_map(g.exportLeaves(), o.exportLeaves(), "wall under misses")
    acc = g.getGrid().getAccessor()
    assert all(acc.isValueOn((x, 5, z)) for x in range(2, 7) for z in (0, 1))
    both(g, o, "restoreMapIntegrity")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "restored")
    both(g, o, "insertPointCloud", ray, (0.0, 5.0, 0.0), "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "after the set is gone")


def test_areas_over_scanned_room_match_oracle(vdbg, oracle):
    wl = W.get("small")
    g, o = pair(vdbg, oracle, wl.resolution, wl.config, wl.max_range)
    rng = np.random.default_rng(17)
    areas = []
    for _ in range(3):
        c = rng.uniform(-15, 15, 2)
        k = int(rng.integers(3, 6))
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        r = rng.uniform(1.0, 6.0, k)
        areas.append([(c[0] + r[j] * np.cos(ang[j]), c[1] + r[j] * np.sin(ang[j]), 0.3, 1.0) for j in range(k)])
    both(g, o, "addArtificialAreas", areas, -0.2, 1.5)
    for k in (0, 1, 0, 2):
        pts, org = wl.scan(k)
        both(g, o, "insertPointCloud", pts[::4], org, "s")
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"areas, scan {k}")
    # replacing the areas restores the old ones first
    both(g, o, "addArtificialAreas", areas[:1], 0.0, 0.5)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "areas replaced")
    pts, org = wl.scan(3)
    both(g, o, "insertPointCloud", pts[::4], org, "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "after replacement")


def test_restore_with_a_negative_threshold_creates_leaves(vdbg, oracle):
    cfg = dataclasses.replace(W.default_config(100.0), prob_thres_max=0.4)
    g, o = pair(vdbg, oracle, 1.0, cfg, 100.0)
    both(g, o, "addArtificialWall", (2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 1.0)
    both(g, o, "restoreMapIntegrity")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "restore creates")
    assert len(g.exportLeaves()[0]) == 1
