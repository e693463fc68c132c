"""GPU parity of map sections (VDBMapping.hpp:922-1085) against the oracle:
extraction over index boxes (full and sparse), applyMapSectionUpdateGrid and
applyMapSectionGrid (with the tiles of the section tree), for a single map
and for a map of a batch. Bit-exact: leaf set, FP32 values as uint32, masks."""
import numpy as np
import pytest

from vdb_mapping_gb300 import workloads as W

from test_gpu_parity import assert_same_map

pytestmark = pytest.mark.gpu


def same_section(a, b, what=""):
    (ao, av, am), (bo, bv, bm) = a, b
    assert ao.shape == bo.shape, (what, ao.shape, bo.shape)
    assert np.array_equal(ao, bo), what
    assert np.array_equal(av.view(np.uint32), bv.view(np.uint32)), what
    assert np.array_equal(am, bm), what


def built_pair(vdbg, oracle):
    wl = W.get("small")
    g = vdbg.OccupancyVDBMapping(wl.resolution)
    o = oracle.OracleMap(wl.resolution)
    for m in (g, o):
        m.setConfig(wl.config)
        m.addInputSource("s", wl.max_range, 0)
    for k in (0, 0, 0, 0, 0, 1, 2):  # repeated hits turn voxels active
        pts, org = wl.scan(k)
        g.insertPointCloud(pts[::4], org, "s")
        o.insertPointCloud(pts[::4], org, "s")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "built maps")
    return g, o


def boxes(seed=3, n=12):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        c = rng.integers(-150, 150, 3)
        half = rng.integers(1, 60, 3)
        out.append((c - half, c + half))
    out.append((np.array([-1000, -1000, -1000]), np.array([1000, 1000, 1000])))  # the whole map
    out.append((np.array([5, 5, 5]), np.array([5, 5, 5])))  # one voxel
    return out


@pytest.mark.parametrize("full", [True, False])
def test_section_extraction_matches_oracle(vdbg, oracle, full):
    g, o = built_pair(vdbg, oracle)
    for lo, hi in boxes():
        same_section(g.getMapSection(lo, hi, full), o.getMapSection(lo, hi, full), f"box {lo} {hi}")


def test_apply_section_states_matches_oracle(vdbg, oracle):
    g, o = built_pair(vdbg, oracle)
    src_g, src_o = built_pair(vdbg, oracle)
    for lo, hi in boxes(seed=5, n=4):
        so, _, sm = src_o.getMapSection(lo + 17, hi + 17, full=False)  # a section of another region
        g.applyMapSectionStates(lo, hi, so, sm)
        o.applyMapSectionStates(lo, hi, so, sm)
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"states box {lo} {hi}")
    # states far from every leaf create leaves at value 0
    far = np.array([[4096, 8, -4096]], np.int32)
    mask = np.zeros((1, 8), np.uint64)
    mask[0, 3] = np.uint64(0x8000000000000001)
    g.applyMapSectionStates((4096, 8, -4096), (4103, 15, -4089), far, mask)
    o.applyMapSectionStates((4096, 8, -4096), (4103, 15, -4089), far, mask)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "far states")


def test_apply_section_values_matches_oracle(vdbg, oracle):
    g, o = built_pair(vdbg, oracle)
    rng = np.random.default_rng(9)
    for lo, hi in boxes(seed=7, n=3):
        so, sv, sm = o.getMapSection(lo, hi, full=True)
        # perturb the values and states (values stay FP32 bit patterns)
        sv = (sv * np.float32(0.5) + rng.standard_normal(sv.shape).astype(np.float32) * (sv != 0)).astype(np.float32)
        sm = sm ^ rng.integers(0, 2**63, sm.shape, dtype=np.uint64)
        g.applyMapSectionValues(so + 8, sv, sm)  # shifted by one leaf: new and existing leaves, tiles
        o.applyMapSectionValues(so + 8, sv, sm)
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"values box {lo} {hi}")
    # an all-background leaf where the map has none creates nothing
    n = len(g.exportLeaves()[0])
    z = (np.array([[8000, 0, 0]], np.int32), np.zeros((1, 512), np.float32), np.zeros((1, 8), np.uint64))
    g.applyMapSectionValues(*z)
    o.applyMapSectionValues(*z)
    assert len(g.exportLeaves()[0]) == n
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "background leaf")


def test_sections_of_a_batch_map(vdbg, oracle):
    wl = W.get("small")
    b = vdbg.MapBatch([0.2, wl.resolution])
    b.setConfig(0, W.default_config(5.0))
    b.setConfig(1, wl.config)
    o = oracle.OracleMap(wl.resolution)
    o.setConfig(wl.config)
    o.addInputSource("s", wl.max_range, 0)
    for k in (0, 0, 0, 0, 0, 1):
        pts, org = wl.scan(k)
        b.insert([pts[::16], pts[::4]], [org, org])
        o.insertPointCloud(pts[::4], org, "s")
    for lo, hi in boxes(seed=11, n=4):
        for full in (True, False):
            same_section(b.getMapSection(1, lo, hi, full), o.getMapSection(lo, hi, full), f"batch box {lo} {hi}")
    so, sv, sm = o.getMapSection(np.array([-60, -60, -10]), np.array([60, 60, 20]), full=True)
    b.applyMapSectionValues(1, so + 16, sv, sm)
    o.applyMapSectionValues(so + 16, sv, sm)
    assert_same_map(b.exportLeaves(1), o.exportLeaves(), "batch values")
    # map 0 of the batch is untouched by map 1's sections
    assert len(b.exportLeaves(0)[0]) > 0
