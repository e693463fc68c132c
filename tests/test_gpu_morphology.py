"""GPU parity of the section morphology (VDBMapping.hpp:1094-1147,
vdbg_section_morphology) against the oracle's voxel-set restatement, and of
applyMapSectionUpdateGrid with smoothing (VDBMapping.hpp:1062-1065). Bit-exact:
leaf origins and masks."""
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
