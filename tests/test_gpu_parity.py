"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle and
the golden fixtures. Integer/bit results must be identical: leaf set, the
512 FP32 log-odds per leaf compared bitwise, and the active masks."""
import os

import numpy as np
import pytest

from vdb_mapping_gb300.mapping import Config

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")


def lo(p):
    import math

    return np.float32(math.log(p) - math.log(1 - p))


def ref_config(max_range=10.0):
    return Config(max_range=max_range, fast_mode=False, prob_hit=0.9, prob_miss=0.1, prob_thres_max=0.51,
                  prob_thres_min=0.49)


def assert_same_map(a, b, what=""):
    oa, va, ma = a
    ob, vb, mb = b
    assert oa.shape == ob.shape, f"{what}: leaf count {oa.shape[0]} vs {ob.shape[0]}"
    assert np.array_equal(oa, ob), f"{what}: leaf origins differ"
    diff = np.nonzero(va.view(np.uint32) != vb.view(np.uint32))
    assert diff[0].size == 0, f"{what}: {diff[0].size} values differ, first leaf {oa[diff[0][0]]} off {diff[1][0]}"
    assert np.array_equal(ma, mb), f"{what}: active masks differ"


def pair(vdbg, oracle, res, cfg, source="s", range_=None, **kw):
    g = vdbg.OccupancyVDBMapping(res, **kw)
    o = oracle.OracleMap(res)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource(source, cfg.max_range if range_ is None else range_, 0)
    return g, o


# --------------------------------------------------------------------------
# The reference's unit tests (tests/mapping.cpp) through the GPU library
# --------------------------------------------------------------------------

def test_set_config(vdbg, capsys):
    m = vdbg.OccupancyVDBMapping(1.0)
    acc = m.getGrid().getAccessor()
    assert m.insertPointCloud(np.array([[0, 0, 1]], np.float32), (0, 0, 0), "test") is True
    assert acc.getValue((0, 0, 1)) == 0.0
    assert "Source not available" in capsys.readouterr().out
    c = ref_config()
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud(np.array([[0, 0, 1]], np.float32), (0, 0, 0), "test")
    assert acc.getValue((0, 0, 0)) == lo(0.1)
    assert acc.getValue((0, 0, 1)) == lo(0.9)


@pytest.mark.parametrize("sign", [1, -1])
def test_insert_axis_point(vdbg, sign):
    res = 0.1
    m = vdbg.OccupancyVDBMapping(res)
    c = ref_config()
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud(np.array([[0, 0, sign * 5 * res]], np.float32), (0, 0, 0), "test")
    acc = m.getGrid().getAccessor()
    for i in range(0 if sign > 0 else 1, 5):
        assert acc.getValue((0, 0, sign * i)) == lo(0.1)
        assert not acc.isValueOn((0, 0, sign * i))
    assert acc.getValue((0, 0, sign * 5)) == lo(0.9)
    assert acc.isValueOn((0, 0, sign * 5))


def test_insert_max_range_point(vdbg):
    res = 0.1
    m = vdbg.OccupancyVDBMapping(res)
    c = ref_config(max_range=0.5)
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud(np.array([[0, 0, 7 * res]], np.float32), (0, 0, 0), "test")
    acc = m.getGrid().getAccessor()
    for i in range(0, int(0.5 / res) + 1):
        assert acc.getValue((0, 0, i)) == lo(0.1)
        assert not acc.isValueOn((0, 0, i))
    assert acc.getValue((0, 0, int(0.5 / res) + 1)) == 0.0
    assert not acc.isValueOn((0, 0, int(0.5 / res) + 1))


def test_reset_map(vdbg):
    m = vdbg.OccupancyVDBMapping(1.0)
    c = ref_config()
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud(np.array([[0, 0, 1]], np.float32), (0, 0, 0), "test")
    acc = m.getGrid().getAccessor()
    assert acc.getValue((0, 0, 1)) == lo(0.9)
    m.resetMap()
    acc = m.getGrid().getAccessor()
    assert acc.getValue((0, 0, 1)) == 0.0
    assert m.leafCount() == 0
    # the map keeps working after a reset
    m.insertPointCloud(np.array([[0, 0, 1]], np.float32), (0, 0, 0), "test")
    assert m.getGrid().getValue((0, 0, 1)) == lo(0.9)


# --------------------------------------------------------------------------
# Golden fixtures
# --------------------------------------------------------------------------

def golden_cases():
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


@pytest.mark.parametrize("name", golden_cases())
def test_golden(vdbg, name):
    from golden_io import load_case, replay

    case = load_case(os.path.join(GOLDEN, name))
    got = replay(vdbg.OccupancyVDBMapping(case["res"]), case)
    assert_same_map(got, (case["origins"], case["values"], case["masks"]), name)


# --------------------------------------------------------------------------
# Against the oracle on seeded workloads
# --------------------------------------------------------------------------

def run_both(g, o, scans, source="s"):
    for pts, org in scans:
        g.insertPointCloud(pts, org, source)
        o.insertPointCloud(pts, org, source)
        for k in ("rays", "visits", "hits", "updates", "new_leaves"):
            assert g.last_stats[k] == o.last_stats[k], (k, g.last_stats, o.last_stats)


def test_small_workload_all_scans(vdbg, oracle):
    from vdb_mapping_gb300 import workloads as W

    w = W.get("small")
    g, o = pair(vdbg, oracle, w.resolution, w.config)
    run_both(g, o, [w.scan(k) for k in range(w.n_scans)])
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "small")


def test_stress_subsample_far_origin(vdbg, oracle):
    from vdb_mapping_gb300 import workloads as W

    w = W.get("stress")
    g, o = pair(vdbg, oracle, w.resolution, w.config)
    scans = []
    for k in range(3):
        p, org = w.scan(k)
        scans.append((p[:3000], org))
    run_both(g, o, scans)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "stress subsample")


def test_dense_first_scan(vdbg, oracle):
    """One full 262,144-point street scan (1.5M leaves): bit-exact."""
    from vdb_mapping_gb300 import workloads as W

    w = W.get("dense")
    g, o = pair(vdbg, oracle, w.resolution, w.config)
    run_both(g, o, [w.scan(0)])
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "dense scan 0")


def test_pool_growth_retry_is_exact(vdbg, oracle):
    """A tiny initial pool forces allocation failures mid-scan, growth and a
    re-marking pass; the result must not change."""
    from vdb_mapping_gb300 import workloads as W

    w = W.get("small")
    g, o = pair(vdbg, oracle, w.resolution, w.config, initial_leaf_capacity=64)
    run_both(g, o, [w.scan(k) for k in range(2)])
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "growth")


def test_block_pool_growth_retry_is_exact(vdbg, oracle):
    """Tiny leaf and block pools force both to grow mid-scan, several times,
    with the block hash rebuilt and failed leaf cells retried."""
    rng = np.random.default_rng(9)
    cfg = Config(max_range=12.0, prob_hit=0.7, prob_miss=0.4, prob_thres_min=0.12, prob_thres_max=0.97)
    g, o = pair(vdbg, oracle, 0.05, cfg, initial_leaf_capacity=16, initial_block_capacity=2)
    scans = []
    for k in range(3):
        org = rng.uniform(-30, 30, 3)
        d = rng.normal(size=(6000, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pts = (org + d * rng.uniform(0.5, 15.0, (6000, 1))).astype(np.float32)
        scans.append((pts, org))
    run_both(g, o, scans)
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "block growth")


def test_device_pointer_input_matches_host(vdbg, oracle):
    import torch

    from vdb_mapping_gb300 import workloads as W

    w = W.get("small")
    p, org = w.scan(3)
    g1, o = pair(vdbg, oracle, w.resolution, w.config)
    g2 = vdbg.OccupancyVDBMapping(w.resolution)
    g2.setConfig(w.config)
    g2.addInputSource("s", w.max_range, 0)
    g1.insertPointCloud(p, org, "s")
    g2.insertPointCloud(torch.from_numpy(p).cuda(), org, "s")
    o.insertPointCloud(p, org, "s")
    assert_same_map(g1.exportLeaves(), g2.exportLeaves(), "device vs host")
    assert_same_map(g1.exportLeaves(), o.exportLeaves(), "vs oracle")
    # (N,3) layout as well
    g3 = vdbg.OccupancyVDBMapping(w.resolution)
    g3.setConfig(w.config)
    g3.addInputSource("s", w.max_range, 0)
    g3.insertPointCloud(np.ascontiguousarray(p[:, :3]), org, "s")
    assert_same_map(g1.exportLeaves(), g3.exportLeaves(), "xyz stride 12")


def test_random_rays_many_resolutions(vdbg, oracle):
    rng = np.random.default_rng(5)
    for res in (0.02, 0.05, 0.1, 0.2, 0.3, 1.0):
        cfg = Config(max_range=rng.uniform(1, 8), prob_hit=0.7, prob_miss=0.4, prob_thres_min=0.12,
                     prob_thres_max=0.97)
        g, o = pair(vdbg, oracle, res, cfg)
        scans = []
        for k in range(3):
            org = rng.uniform(-50, 50, 3)
            pts = (org + rng.normal(0, 3, (2000, 3))).astype(np.float32)
            scans.append((pts, org))
        run_both(g, o, scans)
        assert_same_map(g.exportLeaves(), o.exportLeaves(), f"res {res}")


# --------------------------------------------------------------------------
# API semantics and error paths
# --------------------------------------------------------------------------

def test_sources_and_accumulation_window(vdbg, oracle):
    cfg = ref_config()
    g = vdbg.OccupancyVDBMapping(0.5)
    o = oracle.OracleMap(0.5)
    rng = np.random.default_rng(2)
    for m in (g, o):
        m.setConfig(cfg)
        m.addInputSource("lidar", 0, 0)
        m.addInputSource("depth", 2.0, 0)
    a = rng.uniform(-4, 4, (500, 3)).astype(np.float32)
    b = rng.uniform(-4, 4, (500, 3)).astype(np.float32)
    for m in (g, o):
        m.accumulateUpdate(a, (0, 0, 0), "lidar")
        m.accumulateUpdate(b, (0.3, 0, 0), "depth")
        m.accumulateUpdate(b, (0, 0.2, 0), "lidar")  # same window: deduplicated with `a`
    assert g.leafCount() == 0  # nothing integrated yet
    for m in (g, o):
        m.integrateUpdate()
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "two sources")
    for m in (g, o):
        m.insertPointCloud(a[:100], (1, 1, 1), "depth")
    assert_same_map(g.exportLeaves(), o.exportLeaves(), "after insert")


def test_error_paths(vdbg):
    from vdb_mapping_gb300 import VdbgError

    m = vdbg.OccupancyVDBMapping(0.1)
    pts = np.array([[0, 0, 1]], np.float32)
    assert m.raycastPointCloud(pts, (0, 0, 0), 5.0, "x") is False  # not configured
    c = ref_config()
    m.setConfig(c)
    with pytest.raises(VdbgError):
        m.raycastPointCloud(pts, (0, 0, 0), 5.0, "x")  # unknown source
    m.addInputSource("s", 0, 0)
    with pytest.raises(VdbgError):
        m.addInputSource("s", 0, 0)
    # voxel index beyond 2^23 is reported and leaves the map untouched
    with pytest.raises(VdbgError) as e:
        m.raycastPointCloud(np.array([[1e6, 0, 0]], np.float32), (0, 0, 0), 0.0, "s")
    assert "COORD_RANGE" in str(e.value)
    assert m.leafCount() == 0
    # NaN origin: nothing cast, no error
    m.insertPointCloud(pts, (np.nan, 0, 0), "s")
    assert m.last_stats["rays"] == 0
    # inf point skipped and counted
    m.insertPointCloud(np.array([[0, np.inf, 1], [0, 0, 1]], np.float32), (0, 0, 0), "s")
    assert m.last_stats["rays"] == 1 and m.last_stats["skipped_nonfinite"] == 1
    # empty cloud is fine
    m.insertPointCloud(np.zeros((0, 3), np.float32), (0, 0, 0), "s")
    # bad probability keeps the old log-odds, like the reference
    bad = ref_config()
    bad.prob_hit = 0.3
    m.setConfig(bad)
    assert m.logOdds()["hit"] == lo(0.9)


def test_memory_budget_is_enforced(vdbg):
    from vdb_mapping_gb300 import VdbgError
    from vdb_mapping_gb300 import workloads as W

    w = W.get("small")
    m = vdbg.OccupancyVDBMapping(w.resolution, initial_leaf_capacity=1024, max_device_bytes=64 << 20)
    m.setConfig(w.config)
    m.addInputSource("s", w.max_range, 0)
    p, org = w.scan(0)
    with pytest.raises(VdbgError) as e:
        m.insertPointCloud(p, org, "s")
    assert "OUT_OF_MEMORY" in str(e.value)
    assert m.deviceBytes() <= 64 << 20
