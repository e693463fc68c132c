"""CPU tests of the oracle: pinned against the reference's own unit tests and
against independent pure-Python restatements of the parts those tests leave
open (quantiser, DDA ties and FP64 stepping, log-odds rules, dedup, clipping,
sources). Runs without a GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from vdb_mapping_gb300.mapping import Config

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("VDB_MAPPING_REFERENCE", "/root/reference")


def ref_config(max_range=10.0):
    # The configuration used by every test in the reference's tests/mapping.cpp.
    return Config(max_range=max_range, fast_mode=False, prob_hit=0.9, prob_miss=0.1, prob_thres_max=0.51,
                  prob_thres_min=0.49)


def lo(p):
    return np.float32(math.log(p) - math.log(1 - p))


# --------------------------------------------------------------------------
# The reference's own tests, compiled against the oracle
# --------------------------------------------------------------------------

@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "tests", "mapping.cpp")),
                    reason="reference tree not present on this machine")
def test_reference_unit_tests_pass_against_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={REF}"], check=True)
    res = subprocess.run([os.path.join(REPO, "oracle", "_ref", "mapping_tests")], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "5 tests, 0 failed" in res.stdout


# --------------------------------------------------------------------------
# The same known answers through the Python face of the oracle
# --------------------------------------------------------------------------

def test_insert_before_config_is_noop(oracle):
    m = oracle.OracleMap(1.0)
    m.insertPointCloud([[0, 0, 1]], (0, 0, 0), "test")
    assert m.getValue((0, 0, 1)) == 0.0
    c = ref_config()
    assert m.setConfig(c) == 0
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud([[0, 0, 1]], (0, 0, 0), "test")
    assert m.getValue((0, 0, 0)) == lo(0.1)
    assert m.getValue((0, 0, 1)) == lo(0.9)


@pytest.mark.parametrize("sign", [1, -1])
def test_axis_point(oracle, sign):
    res = 0.1
    m = oracle.OracleMap(res)
    c = ref_config()
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud([[0, 0, sign * 5 * res]], (0, 0, 0), "test")
    for i in range(0 if sign > 0 else 1, 5):
        assert m.getValue((0, 0, sign * i)) == lo(0.1)
        assert not m.isValueOn((0, 0, sign * i))
    assert m.getValue((0, 0, sign * 5)) == lo(0.9)
    assert m.isValueOn((0, 0, sign * 5))


def test_max_range_point_is_free_space(oracle):
    res = 0.1
    m = oracle.OracleMap(res)
    c = ref_config(max_range=0.5)
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud([[0, 0, 7 * res]], (0, 0, 0), "test")
    for i in range(0, int(0.5 / res) + 1):
        assert m.getValue((0, 0, i)) == lo(0.1)
        assert not m.isValueOn((0, 0, i))
    assert m.getValue((0, 0, int(0.5 / res) + 1)) == 0.0


def test_reset(oracle):
    m = oracle.OracleMap(1.0)
    c = ref_config()
    m.setConfig(c)
    m.addInputSource("test", c.max_range, 0)
    m.insertPointCloud([[0, 0, 1]], (0, 0, 0), "test")
    assert m.getValue((0, 0, 1)) == lo(0.9)
    m.resetMap()
    assert m.getValue((0, 0, 1)) == 0.0
    assert m.leafCount() == 0


# --------------------------------------------------------------------------
# Independent restatements (pure Python, IEEE doubles, no FMA)
# --------------------------------------------------------------------------

def py_world_to_index(w, res):
    """VDBMapping.hpp:612-631 with OpenVDB's linear map (w * (1/res))."""
    inv = 1.0 / res
    out = []
    for x in w:
        x = float(x)
        if math.fmod(x, res) != 0.0:
            x = x + res / 2.0
        out.append(math.floor(x * inv))
    return tuple(out)


def py_cast_ray(o, e):
    """castRayIntoGrid (VDBMapping.hpp:550-566) over OpenVDB's DDA<Ray<double>,0>."""
    if tuple(o) == tuple(e):
        return []
    big = 1.7976931348623157e308
    vox, step, nxt, dlt = [0] * 3, [0] * 3, [0.0] * 3, [0.0] * 3
    for a in range(3):
        eye = float(o[a]) + 0.5
        d = float(e[a]) - float(o[a])
        pos = eye + d * 0.0
        vox[a] = math.floor(pos)
        if d == 0.0:
            step[a], nxt[a], dlt[a] = 0, big, big
        else:
            inv = 1.0 / d
            if inv > 0:
                step[a] = 1
                nxt[a] = 0.0 + (float(vox[a] + 1) - pos) * inv
            else:
                step[a] = -1
                nxt[a] = 0.0 + (float(vox[a]) - pos) * inv
            dlt[a] = float(step[a]) * inv
    out = [tuple(vox)]
    while True:
        a = 2
        if nxt[1] < nxt[a]:
            a = 1
        if nxt[0] < nxt[a]:
            a = 0
        t0 = nxt[a]
        nxt[a] += dlt[a]
        vox[a] += step[a]
        if not t0 <= 1.0:
            return out
        out.append(tuple(vox))


@pytest.mark.parametrize("res", [0.1, 0.05, 0.02, 1.0, 0.3, 0.25])
def test_world_to_index_matches_python(oracle, res):
    rng = np.random.default_rng(7)
    vals = list(rng.uniform(-300, 300, 2000))
    # exact multiples, half-way points and their float32 neighbours
    for k in range(-50, 50):
        for base in (k * res, (k - 0.5) * res, (k + 0.5) * res):
            vals.append(base)
            f = np.float32(base)
            vals += [float(f), float(np.nextafter(f, np.float32(np.inf))), float(np.nextafter(f, np.float32(-np.inf)))]
    vals += [0.0, -0.0, 5000.0, -3000.0, 40.0, 1e-9, -1e-9]
    for i in range(0, len(vals) - 2, 3):
        w = vals[i:i + 3]
        assert oracle.world_to_index(res, w) == py_world_to_index(w, res), (w, res)


def test_world_to_index_known_answers(oracle):
    assert oracle.world_to_index(0.1, (0.0, 0.0, float(np.float32(0.5)))) == (0, 0, 5)
    assert oracle.world_to_index(0.1, (0.0, 0.0, float(np.float32(-0.5)))) == (0, 0, -5)
    assert oracle.world_to_index(1.0, (0.0, 0.0, 1.0)) == (0, 0, 1)
    assert oracle.world_to_index(1.0, (-1.0, 2.0, -3.0)) == (-1, 2, -3)
    assert oracle.world_to_index(1.0, (0.49, 0.5, -0.5)) == (0, 1, 0)


def test_dda_known_paths(oracle):
    path = [tuple(v) for v in oracle.cast_ray((0, 0, 0), (0, 0, 5))]
    assert path == [(0, 0, i) for i in range(6)]
    # x/y tie resolved to y, every time
    path = [tuple(v) for v in oracle.cast_ray((0, 0, 0), (3, 3, 0))]
    assert path == [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 2, 0), (2, 2, 0), (2, 3, 0), (3, 3, 0)]
    # three-way tie: z, then y, then x
    path = [tuple(v) for v in oracle.cast_ray((0, 0, 0), (1, 1, 1))]
    assert path == [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1)]
    assert oracle.cast_ray((4, 4, 4), (4, 4, 4)).shape[0] == 0


def test_dda_matches_python_restatement(oracle):
    rng = np.random.default_rng(11)
    cases = []
    for _ in range(1500):
        o = rng.integers(-300000, 300000, 3)
        d = rng.integers(-40, 41, 3)
        cases.append((o, o + d))
    for _ in range(300):
        o = rng.integers(-1000, 1000, 3)
        d = rng.integers(-3000, 3001, 3)
        cases.append((o, o + d))
    # exact-tie families
    for p in [(1, 1, 0), (1, 3, 0), (2, 6, 0), (3, 5, 0), (1, 3, 5), (5, 5, 5), (7, 21, 35), (2, 2, 1)]:
        for s in (1, 3, 7, 40):
            for sg in [(1, 1, 1), (-1, 1, 1), (1, -1, -1), (-1, -1, -1)]:
                d = np.array(p) * s * np.array(sg)
                o = rng.integers(-250000, 250000, 3)
                cases.append((o, o + d))
                cases.append((o, o + d[[2, 0, 1]]))
    for o, e in cases:
        got = [tuple(v) for v in oracle.cast_ray(o, e)]
        want = py_cast_ray(o, e)
        assert got == want, (o, e)
        if want:
            l1 = int(np.abs(np.asarray(e) - np.asarray(o)).sum())
            assert len(want) == l1 + 1
            assert want[-1] == tuple(int(v) for v in e)


def py_update(v, on, hit, c):
    """OccupancyVDBMapping.hpp:92-117 in float32."""
    f = np.float32
    hit_lo, miss_lo = lo(c.prob_hit), lo(c.prob_miss)
    tmin, tmax = lo(c.prob_thres_min), lo(c.prob_thres_max)
    mx, mn = f(math.log(0.99) - math.log(0.01)), f(math.log(0.01) - math.log(0.99))
    if hit:
        v = f(v + hit_lo)
        if v > tmax:
            on = True
            if v > mx:
                v = mx
    else:
        v = f(v + miss_lo)
        if v < tmin:
            on = False
            if v < mn:
                v = mn
    return v, on


@pytest.mark.parametrize("cfg", [
    Config(max_range=10, prob_hit=0.7, prob_miss=0.4, prob_thres_min=0.12, prob_thres_max=0.97),
    Config(max_range=10, prob_hit=0.9, prob_miss=0.1, prob_thres_min=0.49, prob_thres_max=0.51),
    Config(max_range=10, prob_hit=0.6, prob_miss=0.45, prob_thres_min=0.5, prob_thres_max=0.5),
])
def test_repeated_updates_clamp_and_hysteresis(oracle, cfg):
    """Hits and misses on one voxel in sequence follow the float32 rules."""
    m = oracle.OracleMap(1.0)
    m.setConfig(cfg)
    m.addInputSource("s", cfg.max_range, 0)
    seq = [True] * 8 + [False] * 14 + [True] * 3 + [False, True] * 5 + [False] * 30
    v, on = np.float32(0.0), False
    for hit in seq:
        pt = [[0, 0, 3]] if hit else [[0, 0, 5]]  # miss: the ray passes voxel (0,0,3)
        m.insertPointCloud(pt, (0, 0, 0.0), "s")
        v, on = py_update(v, on, hit, cfg)
        assert m.getValue((0, 0, 3)) == v
        assert m.isValueOn((0, 0, 3)) == on


def test_hit_overrides_miss_and_dedup(oracle):
    c = ref_config()
    m = oracle.OracleMap(1.0)
    m.setConfig(c)
    m.addInputSource("s", c.max_range, 0)
    # one ray ends at (0,0,2), another passes through it; three rays share (0,0,1)
    m.insertPointCloud([[0, 0, 2], [0, 0, 4], [0, 0, 3]], (0, 0, 0), "s")
    assert m.getValue((0, 0, 2)) == lo(0.9)
    assert m.getValue((0, 0, 1)) == lo(0.1)
    assert m.last_stats["updates"] == 5  # voxels 0..4 once each
    assert m.last_stats["visits"] == (3 + 1) + (5 + 1) + (4 + 1)


def test_clip_is_strictly_greater(oracle):
    c = ref_config(max_range=2.0)
    m = oracle.OracleMap(1.0)
    m.setConfig(c)
    m.addInputSource("s", c.max_range, 0)
    m.insertPointCloud([[0, 0, 2.0]], (0, 0, 0), "s")  # exactly at max_range: a hit
    assert m.getValue((0, 0, 2)) == lo(0.9)
    m2 = oracle.OracleMap(1.0)
    m2.setConfig(c)
    m2.addInputSource("s", c.max_range, 0)
    m2.insertPointCloud([[0, 0, 2.5]], (0, 0, 0), "s")  # beyond: free space to the clip point
    assert m2.getValue((0, 0, 2)) == lo(0.1)


def test_nan_and_inf_points_are_skipped(oracle):
    c = ref_config()
    m = oracle.OracleMap(1.0)
    m.setConfig(c)
    m.addInputSource("s", c.max_range, 0)
    m.insertPointCloud([[np.nan, 0, 1], [0, np.inf, 1], [0, 0, 1]], (0, 0, 0), "s")
    assert m.last_stats["rays"] == 1
    m.insertPointCloud([[0, 0, 1]], (np.nan, 0, 0), "s")
    assert m.last_stats["rays"] == 0


def test_sources(oracle):
    c = ref_config()
    m = oracle.OracleMap(1.0)
    m.setConfig(c)
    assert m.addInputSource("a", 0, 0) == 0  # range 0 -> configured max_range
    assert m.addInputSource("a", 0, 0) != 0
    assert m.insertPointCloud([[0, 0, 20]], (0, 0, 0), "a") == 0
    assert m.getValue((0, 0, 10)) == lo(0.1)  # clipped at the configured 10 m
    assert m.getValue((0, 0, 11)) == 0.0
    assert m.insertPointCloud([[0, 0, 1]], (0, 0, 0), "nope") != 0
    # two sources accumulate into separate update grids; integration applies both
    m.addInputSource("b", 5, 0)
    m.accumulateUpdate([[1, 0, 0]], (0, 0, 0), "a")
    m.accumulateUpdate([[1, 0, 0]], (0, 0, 0), "b")
    m.integrateUpdate()
    v, on = py_update(*py_update(np.float32(0), False, True, c), True, c)
    assert m.getValue((1, 0, 0)) == v


def test_bad_config_keeps_log_odds(oracle):
    m = oracle.OracleMap(1.0)
    assert m.setConfig(ref_config()) == 0
    bad = ref_config()
    bad.prob_miss = 0.7
    assert m.setConfig(bad) != 0
    assert m.logOdds()["miss"] == lo(0.1)
    neg = ref_config(max_range=-1.0)
    assert m.setConfig(neg) != 0


# --------------------------------------------------------------------------
# Golden fixtures: the committed vectors still come out of the oracle
# --------------------------------------------------------------------------

GOLDEN = os.path.join(REPO, "tests", "golden")


def golden_cases():
    if not os.path.isdir(GOLDEN):
        return []
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_reproduces_golden(oracle, name):
    from golden_io import load_case, run_oracle_case

    case = load_case(os.path.join(GOLDEN, name))
    origins, values, masks = run_oracle_case(oracle, case)
    assert np.array_equal(origins, case["origins"])
    assert np.array_equal(values.view(np.uint32), case["values"].view(np.uint32))
    assert np.array_equal(masks, case["masks"])


def variant_sensitivity(oracle, n_scans):
    """Rays of the stress workload whose quantised endpoint (or clip flag)
    changes under each arithmetic variant of the unpinned OpenVDB facts; a ray
    whose origin and end voxels agree walks the same DDA path, so these rays
    bound every voxel the variants could change."""
    from vdb_mapping_gb300 import workloads as W

    w = W.get("stress")
    out = {"rays": 0, "origin_voxels_differ": {}, "w2i_divide": 0, "unit_reciprocal": 0}
    for k in range(n_scans):
        pts, org = w.scan(k)
        base = oracle.clip_quantise(pts, org, w.max_range, w.resolution)
        out["rays"] += int(base[:, 0].sum())
        for name, kw in (("w2i_divide", {"w2i_divide": True}), ("unit_reciprocal", {"unit_reciprocal": True})):
            rec = oracle.clip_quantise_variant(pts, org, w.max_range, w.resolution, **kw)
            out[name] += int(np.count_nonzero(np.any(rec != base, axis=1)))
            o1 = oracle.world_to_index(w.resolution, org)
            o2 = oracle.world_to_index(w.resolution, org, divide=True)
            out["origin_voxels_differ"][k] = o1 != o2
    return out


def test_variant_sensitivity_on_stress_workload(oracle):
    # The default reading (multiply by 1/res, unit() by division) is the one
    # the reference's own tests pin and the GPU path implements; the counts
    # say how many stress-config rays the two unpinned readings would move.
    s = variant_sensitivity(oracle, 20)
    assert s["rays"] > 1_000_000
    assert s["w2i_divide"] >= 0 and s["unit_reciprocal"] >= 0
    print("stress variant sensitivity:", s)
