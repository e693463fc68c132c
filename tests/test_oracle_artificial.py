"""Known answers for the oracle's artificial areas (VDBMapping.hpp:1152-1236
and the re-activation in updateMap, :785-789). The reference has no tests
for them; the answers follow its code: walls are castRayIntoGrid lines per
layer, their voxels are set active after every non-empty update, and
restoreMapIntegrity gives them back the state their value implies.
1 m voxels, so index = world."""
import dataclasses

import numpy as np

from vdb_mapping_gb300 import workloads as W

WALL = [(x, 5, z) for z in (0, 1) for x in range(2, 7)]


def fresh(oracle, cfg=None):
    m = oracle.OracleMap(1.0)
    assert m.setConfig(cfg or W.default_config(100.0)) == 0
    m.addInputSource("s", 100.0, 0)
    return m


def active(m, voxels):
    return [m.isValueOn(v) for v in voxels]


def test_wall_voxels_turn_active_with_the_next_update(oracle):
    m = fresh(oracle)
    m.addArtificialWall((2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 2.0)
    assert m.leafCount() == 0  # nothing happens before an update
    m.insertPointCloud(np.array([[0.0, 0.0, 3.0]], np.float32), (0.0, 0.0, 0.0), "s")
    assert all(active(m, WALL))
    assert m.getValue((4, 5, 1)) == 0.0  # the background value
    assert not m.isValueOn((7, 5, 0)) and not m.isValueOn((4, 5, 2))


def test_an_empty_update_does_not_reactivate(oracle):
    m = fresh(oracle)
    m.addArtificialWall((2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 2.0)
    m.integrateUpdate()  # no data accumulated: updateMap returns early
    assert m.leafCount() == 0


def test_misses_cannot_clear_the_wall_until_restored(oracle):
    m = fresh(oracle)
    m.addArtificialWall((2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 2.0)
    miss = m.logOdds()["miss"]
    ray = np.array([[10.0, 5.0, 0.0]], np.float32)
    for _ in range(6):  # enough misses to fall below the lower threshold
        m.insertPointCloud(ray, (0.0, 5.0, 0.0), "s")
    assert all(active(m, WALL))
    assert m.getValue((3, 5, 0)) < 5 * miss < 0.0
    m.restoreMapIntegrity()
    # value <= thres_max: inactive; the untouched layer (value 0) too
    assert not any(active(m, WALL))
    m.insertPointCloud(ray, (0.0, 5.0, 0.0), "s")
    assert not any(active(m, WALL))  # the set is gone


def test_polygon_and_areas(oracle):
    m = fresh(oracle)
    square = [(10.0, 10.0, 0.0, 1.0), (13.0, 10.0, 0.0, 1.0), (13.0, 13.0, 0.0, 1.0), (10.0, 13.0, 0.0, 1.0)]
    m.addArtificialAreas([square], 0.0, 1.0)
    m.insertPointCloud(np.array([[0.0, 0.0, 3.0]], np.float32), (0.0, 0.0, 0.0), "s")
    ring = {(x, y, 0) for x in range(10, 14) for y in range(10, 14)} - {(11, 11, 0), (12, 11, 0), (11, 12, 0),
                                                                       (12, 12, 0)}
    for x in range(9, 15):
        for y in range(9, 15):
            assert m.isValueOn((x, y, 0)) == ((x, y, 0) in ring), (x, y)
    # replacing the areas restores the old ring first
    m.addArtificialAreas([], 0.0, 1.0)
    assert not any(m.isValueOn(v) for v in ring)


def test_restore_creates_leaves_when_the_background_exceeds_the_threshold(oracle):
    cfg = dataclasses.replace(W.default_config(100.0), prob_thres_max=0.4)  # log-odds below 0
    m = fresh(oracle, cfg)
    m.addArtificialWall((2.0, 5.0, 0.0), (6.0, 5.0, 0.0), 0.0, 1.0)
    m.restoreMapIntegrity()
    assert all(m.isValueOn((x, 5, 0)) for x in range(2, 7))
