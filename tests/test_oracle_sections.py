"""Known answers for the oracle's map-section restatement (VDBMapping.hpp:
getMapSection 922-1012, applyMapSectionGrid 1022-1048,
applyMapSectionUpdateGrid 1058-1085). The reference has no tests for these;
the answers below follow OpenVDB's accessor rules as stated in the oracle."""
import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W


def vdb_off(x, y, z):
    return ((x & 7) << 6) | ((y & 7) << 3) | (z & 7)


def small_map(oracle):
    """Five scans of three rays from the origin (0.1 m voxels): the end voxels
    (20,0,0), (20,4,0) and (0,0,12) turn active, the voxels before them hold
    miss log-odds."""
    m = oracle.OracleMap(0.1)
    assert m.setConfig(W.default_config(10.0)) == 0
    m.addInputSource("s", 10.0, 0)
    pts = np.array([[2.0, 0.0, 0.0], [2.0, 0.4, 0.0], [0.0, 0.0, 1.2]], np.float32)
    for _ in range(5):
        m.insertPointCloud(pts, (0.0, 0.0, 0.0), "s")
    return m


def test_section_full_and_sparse(oracle):
    m = small_map(oracle)
    o, v, mk = m.exportLeaves()
    lo, hi = (3, -1, -1), (12, 2, 2)
    so, sv, sm = m.getMapSection(lo, hi, full=True)
    # the leaves overlapping [3, 12] in x that hold voxels inside the box
    assert sorted(map(tuple, so)) == [(0, 0, 0), (8, 0, 0)]
    for k, org in enumerate(so):
        i = [tuple(x) for x in o].index(tuple(org))
        for x in range(8):
            for y in range(8):
                for z in range(8):
                    c = (org[0] + x, org[1] + y, org[2] + z)
                    off = vdb_off(*c)
                    inside = all(lo[a] <= c[a] <= hi[a] for a in range(3))
                    bit = (int(sm[k][off >> 6]) >> (off & 63)) & 1
                    mbit = (int(mk[i][off >> 6]) >> (off & 63)) & 1
                    assert sv[k][off] == (v[i][off] if inside else 0.0)
                    assert bit == (mbit if inside else 0)
    po, pv, pm = m.getMapSection(lo, hi, full=False)
    for k in range(len(po)):
        on = np.array([(int(pm[k][off >> 6]) >> (off & 63)) & 1 for off in range(512)], bool)
        assert np.all(pv[k][on] == 1.0) and np.all(pv[k][~on] == 0.0)
    # a box holding only inactive zero voxels yields no leaf
    eo, _, _ = m.getMapSection((0, 5, 5), (7, 7, 7), full=True)
    assert len(eo) == 0


def test_apply_section_states(oracle):
    m = small_map(oracle)
    n_before = m.activeVoxelCount()
    lo, hi = (0, 0, 0), (30, 7, 7)
    so, _, sm = m.getMapSection(lo, hi, full=False)
    t = small_map(oracle)
    # deactivates everything inside the box, then restores the same states
    t.applyMapSectionStates(lo, hi, so, sm)
    assert t.activeVoxelCount() == n_before
    # an empty section clears the box
    t.applyMapSectionStates(lo, hi, np.zeros((0, 3), np.int32), np.zeros((0, 8), np.uint64))
    _, _, km = t.getMapSection(lo, hi, full=False)
    assert len(km) == 0
    # a state outside the map's leaves creates a leaf at background 0
    far = np.array([[800, 800, 800]], np.int32)
    mask = np.zeros((1, 8), np.uint64)
    mask[0][0] = np.uint64(1)
    t.applyMapSectionStates((800, 800, 800), (800, 800, 800), far, mask)
    assert t.isValueOn((800, 800, 800)) and t.getValue((800, 800, 800)) == 0.0


def test_apply_section_values_and_tiles(oracle):
    m = small_map(oracle)
    assert m.isValueOn((20, 0, 0))  # the hit at x = 2.0 m
    # section: the leaf at the origin only, every voxel set to 0.5 and on
    org = np.array([[0, 0, 0]], np.int32)
    vals = np.full((1, 512), 0.5, np.float32)
    masks = np.full((1, 8), np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    before = m.leafCount()
    m.applyMapSectionValues(org, vals, masks)
    assert m.getValue((3, 5, 7)) == 0.5 and m.isValueOn((3, 5, 7))
    # the empty slot (8,0,0) of the section's 128^3 node is a tile: the map
    # voxel at that origin becomes inactive background, the rest of its leaf stays
    assert m.getValue((8, 0, 0)) == 0.0 and not m.isValueOn((8, 0, 0))
    assert m.getValue((9, 0, 0)) != 0.0
    # (16,0,0) .. (120,0,0) likewise; (20,0,0) is not a slot origin and keeps its state
    assert m.isValueOn((20, 0, 0))
    assert m.leafCount() == before
    # an all-background leaf where the map has none creates nothing
    m.applyMapSectionValues(np.array([[4000, 0, 0]], np.int32), np.zeros((1, 512), np.float32),
                            np.zeros((1, 8), np.uint64))
    assert m.leafCount() == before


@pytest.mark.parametrize("full", [True, False])
def test_section_round_trip_on_small_scans(oracle, full):
    wl = W.get("small")
    m = oracle.OracleMap(wl.resolution)
    m.setConfig(wl.config)
    m.addInputSource("s", wl.max_range, 0)
    pts, org = wl.scan(0)
    for _ in range(5):  # repeated hits turn voxels active
        m.insertPointCloud(pts[::8], org, "s")
    lo, hi = (-40, -30, -5), (25, 35, 12)
    so, sv, sm = m.getMapSection(lo, hi, full=full)
    assert len(so) > 0
    # applying a sparse section's states to the same map changes nothing
    n = m.activeVoxelCount()
    m.applyMapSectionStates(lo, hi, so, sm)
    assert m.activeVoxelCount() == n


def test_create_index_bounding_box():
    from vdb_mapping_gb300 import createIndexBoundingBox
    eye = np.eye(4)
    lo, hi = createIndexBoundingBox((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), eye, 0.1)
    assert tuple(lo) == (0, 0, 0) and tuple(hi) == (10, 10, 10)
    lo, hi = createIndexBoundingBox((-0.25, 0.0, 0.0), (0.25, 2.0, 0.5), eye, 0.1)
    assert tuple(lo) == (-3, 0, 0) and tuple(hi) == (2, 20, 5)
    rot = np.array([[0, -1, 0, 1.0], [1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], np.float64)  # 90 deg about z, +1 m x
    lo, hi = createIndexBoundingBox((0.0, 0.0, 0.0), (1.0, 2.0, 1.0), rot, 0.5)
    assert tuple(lo) == (-2, 0, 0) and tuple(hi) == (2, 2, 2)


def test_apply_smoothed_value_section(oracle):
    """applyMapSectionGrid with smoothing (VDBMapping.hpp:1026-1029): the
    closing fills the gap between two active voxels with the section's stored
    value there, and the leaves its dilation reached are written as well: a
    leaf the erosion emptied again overwrites the map leaf there with
    inactive zeros (the morphology does not prune it)."""
    m = small_map(oracle)
    assert m.getValue((-1, 0, 0)) == 0.0
    # a map leaf at (-8, 0, 0) with values: a ray towards -x
    m.insertPointCloud(np.array([[-0.75, 0.05, 0.05]], np.float32), (0.0, 0.0, 0.0), "s")
    assert m.getValue((-3, 0, 0)) != 0.0
    org = np.array([[0, 0, 0]], np.int32)
    vals = np.full((1, 512), 0.5, np.float32)
    masks = np.zeros((1, 8), np.uint64)
    for x in (0, 2):
        masks[0][vdb_off(x, 0, 0) >> 6] |= np.uint64(1) << np.uint64(vdb_off(x, 0, 0) & 63)
    unsmoothed = small_map(oracle)
    unsmoothed.insertPointCloud(np.array([[-0.75, 0.05, 0.05]], np.float32), (0.0, 0.0, 0.0), "s")
    unsmoothed.applyMapSectionValues(org, vals, masks)
    assert not unsmoothed.isValueOn((1, 0, 0))
    assert unsmoothed.getValue((-3, 0, 0)) == m.getValue((-3, 0, 0))
    m.applyMapSectionValues(org, vals, masks, smooth=True, iterations=1)
    assert m.isValueOn((1, 0, 0)) and m.getValue((1, 0, 0)) == 0.5
    assert m.isValueOn((0, 0, 0)) and m.isValueOn((2, 0, 0))
    # the dilated, then emptied, leaf (-8, 0, 0) of the section
    assert m.getValue((-3, 0, 0)) == 0.0 and not m.isValueOn((-3, 0, 0))
