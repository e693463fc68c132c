"""GPU parity of the section morphology (VDBMapping.hpp:1094-1147,
vdbg_section_morphology, with and without the kept leaf topology) against the
oracle's voxel-set restatement, and of applyMapSectionUpdateGrid and
applyMapSectionGrid with smoothing (VDBMapping.hpp:1062-1065, 1026-1029).
Bit-exact: leaf origins, masks and values."""
import numpy as np
import pytest

from test_gpu_parity import assert_same_map
from test_gpu_sections import built_pair

pytestmark = pytest.mark.gpu


def random_section(seed, n_leaves, density):
    rng = np.random.default_rng(seed)
    c = rng.integers(-3000, 3000, 3) & ~7
    origins = np.unique(c + 8 * rng.integers(-4, 5, (n_leaves, 3)), axis=0).astype(np.int32)
    bits = rng.random((len(origins), 8, 64)) < density
    masks = (bits * (np.uint64(1) << np.arange(64, dtype=np.uint64))).sum(axis=2, dtype=np.uint64)
    return origins, masks


@pytest.mark.parametrize("op", ["dilate", "erode", "close", "open"])
def test_morphology_matches_oracle(vdbg, oracle, op):
    g = vdbg.OccupancyVDBMapping(0.1)
    for seed in range(6):
        for density in (0.02, 0.3, 0.9):
            o, m = random_section(seed, 40, density)
            it = 1 + seed % 3
            go, gm = g.sectionMorphology(o, m, op, it)
            oo, om = oracle.morphology(o, m, op, it)
            assert np.array_equal(go, oo), (op, seed, density, len(go), len(oo))
            assert np.array_equal(gm, om), (op, seed, density)


def test_morphology_of_an_empty_section(vdbg):
    g = vdbg.OccupancyVDBMapping(0.1)
    o, m = g.sectionMorphology(np.zeros((0, 3), np.int32), np.zeros((0, 8), np.uint64), "close", 2)
    assert len(o) == 0 and len(m) == 0


def test_smoothed_section_states_match_oracle(vdbg, oracle):
    g, o = built_pair(vdbg, oracle)
    src_g, src_o = built_pair(vdbg, oracle)
    lo, hi = np.array([-80, -80, -10]), np.array([80, 80, 20])
    so, _, sm = src_o.getMapSection(lo, hi, full=False)
    g.applyMapSectionStates(lo, hi, so, sm, smooth=True, iterations=2)
    co, cm = oracle.morphology(so, sm, "close", 2)
    o.applyMapSectionStates(lo, hi, co, cm)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "smoothed states")
    assert len(co) >= len(so)


@pytest.mark.parametrize("op", ["dilate", "erode", "close", "open"])
def test_morphology_keeping_leaves_matches_oracle(vdbg, oracle, op):
    g = vdbg.OccupancyVDBMapping(0.1)
    for seed in range(4):
        for density in (0.0, 0.02, 0.5):
            o, m = random_section(100 + seed, 30, density)
            it = 1 + seed % 3
            go, gm = g.sectionMorphology(o, m, op, it, keep_leaves=True)
            oo, om = oracle.morphology(o, m, op, it, keep_leaves=True)
            assert np.array_equal(go, oo), (op, seed, density, len(go), len(oo))
            assert np.array_equal(gm, om), (op, seed, density)
            assert len(go) >= len(o)


@pytest.mark.parametrize("iterations", [1, 2])
def test_smoothed_value_section_matches_oracle(vdbg, oracle, iterations):
    g, o = built_pair(vdbg, oracle)
    _, src_o = built_pair(vdbg, oracle)
    lo, hi = np.array([-60, -60, -8]), np.array([60, 60, 16])
    so, sv, sm = src_o.getMapSection(lo, hi, full=True)
    g.applyMapSectionValues(so, sv, sm, smooth=True, iterations=iterations)
    o.applyMapSectionValues(so, sv, sm, smooth=True, iterations=iterations)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "smoothed values")
    co, _, _ = oracle.close_value_section(so, sv, sm, iterations)
    assert len(co) > len(so)
