"""Known answers for the oracle's morphology (openvdb::tools::dilateActiveValues
/ erodeActiveValues with NN_FACE_EDGE_VERTEX, VDBMapping.hpp:1094-1147), which
applyMapSectionUpdateGrid's smoothing (VDBMapping.hpp:1062-1065) closes the
section with. Voxels are given in index coordinates; leaves in OpenVDB's order."""
import itertools

import numpy as np


def leaves_of(voxels):
    d = {}
    for x, y, z in voxels:
        o = (x & ~7, y & ~7, z & ~7)
        off = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7)
        d.setdefault(o, np.zeros(8, np.uint64))[off >> 6] |= np.uint64(1) << np.uint64(off & 63)
    keys = sorted(d)
    return np.array(keys, np.int32).reshape(-1, 3), np.array([d[k] for k in keys], np.uint64).reshape(-1, 8)


def voxels_of(origins, masks):
    out = set()
    for o, m in zip(origins, masks):
        for off in range(512):
            if (int(m[off >> 6]) >> (off & 63)) & 1:
                out.add((int(o[0]) + (off >> 6), int(o[1]) + ((off >> 3) & 7), int(o[2]) + (off & 7)))
    return out


def cube(c, r):
    return {(c[0] + i, c[1] + j, c[2] + k) for i, j, k in itertools.product(range(-r, r + 1), repeat=3)}


def run(oracle, voxels, op, it):
    return voxels_of(*oracle.morphology(*leaves_of(voxels), op, it))


def test_dilating_one_voxel_gives_its_box_across_leaves(oracle):
    assert run(oracle, [(0, 0, 0)], "dilate", 1) == cube((0, 0, 0), 1)
    assert run(oracle, [(0, 0, 0)], "dilate", 2) == cube((0, 0, 0), 2)
    o, _ = oracle.morphology(*leaves_of([(0, 0, 0)]), "dilate", 1)
    assert len(o) == 8  # the box spans the eight leaves around the origin


def test_eroding_removes_what_has_an_inactive_neighbour(oracle):
    assert run(oracle, [(5, 5, 5)], "erode", 1) == set()
    assert run(oracle, cube((20, -3, 7), 2), "erode", 1) == cube((20, -3, 7), 1)


def test_closing_fills_a_gap_and_keeps_a_point(oracle):
    assert run(oracle, [(0, 0, 0), (2, 0, 0)], "close", 1) == {(0, 0, 0), (1, 0, 0), (2, 0, 0)}
    assert run(oracle, [(9, 9, 9)], "close", 2) == {(9, 9, 9)}


def test_opening_removes_specks_and_keeps_boxes(oracle):
    box = cube((-12, 4, 30), 1)
    assert run(oracle, box | {(40, 40, 40)}, "open", 1) == box


def test_result_is_sorted_and_without_empty_leaves(oracle):
    o, m = oracle.morphology(*leaves_of([(0, 0, 0), (100, 0, 0), (-50, 8, 3)]), "close", 1)
    keys = [tuple(x) for x in o]
    assert keys == sorted(keys)
    assert all(int(np.bitwise_or.reduce(row)) != 0 for row in m)


def test_keep_leaves_holds_every_leaf_a_dilation_reached(oracle):
    # A voxel at a leaf corner: the dilation reaches the seven leaves around
    # it, the erosion empties them again; with the topology kept they stay.
    vox = [(0, 0, 0), (0, 0, 2)]
    o, m = oracle.morphology(*leaves_of(vox), "close", 1, keep_leaves=True)
    assert sorted(map(tuple, o)) == sorted(itertools.product((-8, 0), repeat=3))
    assert voxels_of(o, m) == {(0, 0, 0), (0, 0, 1), (0, 0, 2)}
    assert sum(int(np.bitwise_or.reduce(row)) == 0 for row in m) == 7
    # an empty input leaf stays; erosion alone removes no leaf
    eo = np.array([[64, 64, 64], [0, 0, 0]], np.int32)
    em = np.zeros((2, 8), np.uint64)
    em[1][0] = np.uint64(1)  # voxel (0, 0, 0)
    ko, km = oracle.morphology(eo, em, "erode", 2, keep_leaves=True)
    assert sorted(map(tuple, ko)) == [(0, 0, 0), (64, 64, 64)] and not km.any()
    assert len(oracle.morphology(eo, em, "erode", 2)[0]) == 0


def test_close_value_section_keeps_values_and_zero_fills_new_leaves(oracle):
    o, m = leaves_of([(0, 0, 0), (2, 0, 0)])
    v = np.full((1, 512), 0.25, np.float32)
    co, cv, cm = oracle.close_value_section(o, v, m, 1)
    assert len(co) == 8
    for org, vals in zip(co, cv):
        assert np.all(vals == (0.25 if tuple(org) == (0, 0, 0) else 0.0))
    assert voxels_of(co, cm) == {(0, 0, 0), (1, 0, 0), (2, 0, 0)}
