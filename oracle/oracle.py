"""ctypes face of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline legs, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    lib = C.CDLL(LIB)
    P, D, I64, U64P = C.c_void_p, C.c_double, C.c_int64, C.POINTER(C.c_uint64)
    sig = {
        "vo_create": (P, [D, C.c_int, C.c_int]),
        "vo_destroy": (None, [P]),
        "vo_set_config": (C.c_int, [P, D, C.c_int, D, D, D, D, D]),
        "vo_add_source": (C.c_int, [P, C.c_char_p, D, D]),
        "vo_insert": (C.c_int, [P, P, I64, I64, C.POINTER(D), C.c_char_p, U64P]),
        "vo_accumulate": (C.c_int, [P, P, I64, I64, C.POINTER(D), C.c_char_p, U64P]),
        "vo_integrate": (None, [P, U64P]),
        "vo_reset": (None, [P]),
        "vo_leaf_count": (I64, [P]),
        "vo_active_count": (I64, [P]),
        "vo_export": (None, [P, P, P, P]),
        "vo_change_count": (I64, [P]),
        "vo_export_changes": (None, [P, P, P, P]),
        "vo_get_value": (C.c_float, [P, C.c_int32, C.c_int32, C.c_int32]),
        "vo_is_value_on": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32]),
        "vo_log_odds": (None, [P, C.POINTER(C.c_float)]),
        "vo_cast_ray": (I64, [P, P, P, I64]),
        "vo_world_to_index": (None, [D, C.POINTER(D), P, C.c_int]),
        "vo_clip_quantise": (None, [P, I64, I64, C.POINTER(D), D, D, P]),
        "vo_clip_quantise_variant": (None, [P, I64, I64, C.POINTER(D), D, D, C.c_int, C.c_int, P]),
        "vo_bench_replicas": (D, [D, C.POINTER(D), P, I64, I64, I64, C.POINTER(D), C.c_int, U64P]),
        "vo_section": (I64, [P, P, P, C.c_int, I64, P, P, P]),
        "vo_apply_section_states": (None, [P, P, P, I64, P, P]),
        "vo_apply_section_values": (None, [P, I64, P, P, P]),
        "vo_raytrace": (C.c_int, [P, I64, P, P, P, P, P]),
        "vo_morphology": (I64, [I64, P, P, C.c_int, C.c_int, I64, P, P]),
        "vo_close_value_section": (I64, [I64, P, P, P, C.c_int, I64, P, P, P]),
        "vo_add_artificial_wall": (None, [P, C.POINTER(D), C.POINTER(D), D, D]),
        "vo_restore_map_integrity": (None, [P]),
        "vo_ray_digests": (None, [P, I64, I64, C.POINTER(D), D, D, C.c_int, P]),
        "vo_map_digest": (None, [P, U64P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


STAT_KEYS = ("rays", "visits", "hits", "updates", "new_leaves")


def _cloud(cloud):
    arr = np.asarray(cloud, dtype=np.float32)
    if arr.ndim != 2 or arr.shape[1] < 3:
        raise ValueError("cloud must be (N, 3+)")
    arr = np.ascontiguousarray(arr)
    return arr, arr.shape[0], arr.shape[1]


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


class OracleMap:
    """OccupancyVDBMapping semantics on the CPU (see vdb_oracle.hpp)."""

    def __init__(self, resolution, w2i_divide=False, unit_reciprocal=False):
        self._l = load()
        self._h = self._l.vo_create(float(resolution), int(w2i_divide), int(unit_reciprocal))
        self.resolution = float(resolution)
        self.last_stats = None

    def __del__(self):
        try:
            self._l.vo_destroy(self._h)
        except Exception:
            pass

    def setConfig(self, c) -> int:
        return self._l.vo_set_config(self._h, c.max_range, int(c.fast_mode), c.accumulation_period,
                                     c.prob_hit, c.prob_miss, c.prob_thres_min, c.prob_thres_max)

    def addInputSource(self, sid, max_range, max_rate) -> int:
        return self._l.vo_add_source(self._h, sid.encode(), float(max_range), float(max_rate))

    def _call(self, fn, cloud, origin, sid):
        arr, n, stride = _cloud(cloud)
        st = (C.c_uint64 * 5)()
        r = fn(self._h, arr.ctypes.data, n, stride, _d3(origin), sid.encode(), st)
        self.last_stats = dict(zip(STAT_KEYS, list(st)))
        return r

    def insertPointCloud(self, cloud, origin, sid) -> int:
        return self._call(self._l.vo_insert, cloud, origin, sid)

    def accumulateUpdate(self, cloud, origin, sid) -> int:
        return self._call(self._l.vo_accumulate, cloud, origin, sid)

    def integrateUpdate(self):
        st = (C.c_uint64 * 5)()
        self._l.vo_integrate(self._h, st)
        self.last_stats = dict(zip(STAT_KEYS, list(st)))

    def resetMap(self):
        self._l.vo_reset(self._h)

    def leafCount(self) -> int:
        return self._l.vo_leaf_count(self._h)

    def activeVoxelCount(self) -> int:
        return self._l.vo_active_count(self._h)

    def mapDigest(self):
        """(leaves, voxels, leaf sum, voxel sum), the map digest the library's
        vdbg_map_digest computes."""
        out = (C.c_uint64 * 4)()
        self._l.vo_map_digest(self._h, out)
        return tuple(int(v) for v in out)

    def exportLeaves(self):
        n = self.leafCount()
        origins = np.zeros((n, 3), np.int32)
        values = np.zeros((n, 512), np.float32)
        masks = np.zeros((n, 8), np.uint64)
        self._l.vo_export(self._h, origins.ctypes.data, values.ctypes.data, masks.ctypes.data)
        return origins, values, masks

    def exportChanges(self):
        """Change grid of the last integration: (origins (L,3), active (L,8), value (L,8))."""
        n = self._l.vo_change_count(self._h)
        origins = np.zeros((n, 3), np.int32)
        active = np.zeros((n, 8), np.uint64)
        value = np.zeros((n, 8), np.uint64)
        self._l.vo_export_changes(self._h, origins.ctypes.data, active.ctypes.data, value.ctypes.data)
        return origins, active, value

    def getMapSection(self, lo, hi, full=False):
        """getMapSection over the index box [lo, hi]: (origins, values, masks) sorted by origin."""
        lo = np.ascontiguousarray(lo, np.int32)
        hi = np.ascontiguousarray(hi, np.int32)
        n = self._l.vo_section(self._h, lo.ctypes.data, hi.ctypes.data, 1 if full else 0, 0, None, None, None)
        origins = np.zeros((n, 3), np.int32)
        values = np.zeros((n, 512), np.float32)
        masks = np.zeros((n, 8), np.uint64)
        self._l.vo_section(self._h, lo.ctypes.data, hi.ctypes.data, 1 if full else 0, n, origins.ctypes.data,
                           values.ctypes.data, masks.ctypes.data)
        return origins, values, masks

    def applyMapSectionStates(self, lo, hi, origins, masks):
        """applyMapSectionUpdateGrid over the index box [lo, hi]."""
        lo = np.ascontiguousarray(lo, np.int32)
        hi = np.ascontiguousarray(hi, np.int32)
        o = np.ascontiguousarray(origins, np.int32)
        mk = np.ascontiguousarray(masks, np.uint64)
        self._l.vo_apply_section_states(self._h, lo.ctypes.data, hi.ctypes.data, len(o), o.ctypes.data, mk.ctypes.data)

    def applyMapSectionValues(self, origins, values, masks, smooth=False, iterations=2):
        """applyMapSectionGrid; smooth closes the section first (VDBMapping.hpp:1026-1029)."""
        if smooth:
            origins, values, masks = close_value_section(origins, values, masks, iterations)
        o = np.ascontiguousarray(origins, np.int32)
        v = np.ascontiguousarray(values, np.float32)
        mk = np.ascontiguousarray(masks, np.uint64)
        self._l.vo_apply_section_values(self._h, len(o), o.ctypes.data, v.ctypes.data, mk.ctypes.data)

    def addArtificialWall(self, start, end, negative_height, positive_height):
        """addArtificialWall (VDBMapping.hpp:1210-1236)."""
        self._l.vo_add_artificial_wall(self._h, _d3(start[:3]), _d3(end[:3]), float(negative_height),
                                       float(positive_height))

    def addArtificialPolygon(self, polygon, negative_height, positive_height):
        """addArtificialPolygon (VDBMapping.hpp:1198-1207): walls between consecutive corners, closed."""
        for i in range(len(polygon)):
            self.addArtificialWall(polygon[i], polygon[(i + 1) % len(polygon)], negative_height, positive_height)

    def addArtificialAreas(self, areas, negative_height, positive_height):
        """addArtificialAreas (VDBMapping.hpp:1175-1189): restore, then every polygon."""
        self.restoreMapIntegrity()
        for poly in areas:
            self.addArtificialPolygon(poly, negative_height, positive_height)

    def restoreMapIntegrity(self):
        """restoreMapIntegrity (VDBMapping.hpp:1153-1166)."""
        self._l.vo_restore_map_integrity(self._h)

    def raytrace(self, origins, directions, max_lengths):
        """raytrace (VDBMapping.hpp:675-721): (status, success bool[n], end points [n][3])."""
        o = np.ascontiguousarray(np.asarray(origins, np.float64).reshape(-1, 3))
        d = np.ascontiguousarray(np.asarray(directions, np.float64).reshape(-1, 3))
        n = o.shape[0]
        ln = np.ascontiguousarray(np.broadcast_to(np.asarray(max_lengths, np.float64), (n,)))
        ok = np.zeros(n, np.uint8)
        ends = np.zeros((n, 3), np.float64)
        r = self._l.vo_raytrace(self._h, n, o.ctypes.data, d.ctypes.data, ln.ctypes.data, ok.ctypes.data,
                                ends.ctypes.data)
        return r, ok.astype(bool), ends

    def getValue(self, xyz) -> float:
        return self._l.vo_get_value(self._h, *[int(c) for c in xyz])

    def isValueOn(self, xyz) -> bool:
        return bool(self._l.vo_is_value_on(self._h, *[int(c) for c in xyz]))

    def logOdds(self):
        out = (C.c_float * 2)()
        self._l.vo_log_odds(self._h, out)
        return {"hit": out[0], "miss": out[1]}


def cast_ray(o, e, cap=1 << 20):
    """Voxels castRayIntoGrid visits from voxel o to voxel e, in order."""
    lib = load()
    oo = np.asarray(o, np.int32)
    ee = np.asarray(e, np.int32)
    out = np.zeros((cap, 3), np.int32)
    n = lib.vo_cast_ray(oo.ctypes.data, ee.ctypes.data, out.ctypes.data, cap)
    if n > cap:
        return cast_ray(o, e, cap=int(n))
    return out[:n].copy()


def ray_digests(cloud, origin, max_range, res, threads=None):
    """uint64 (N, 2) per-point traversal digests (the definition of the
    library's vdbg_ray_digests), from the oracle's clip, quantiser and DDA."""
    import os

    arr, n, stride = _cloud(cloud)
    out = np.zeros((n, 2), np.uint64)
    load().vo_ray_digests(arr.ctypes.data, n, stride, _d3(origin), float(max_range), float(res),
                          int(threads or os.cpu_count() or 1), out.ctypes.data)
    return out


def world_to_index(res, w, divide=False):
    lib = load()
    out = np.zeros(3, np.int32)
    lib.vo_world_to_index(float(res), _d3(w), out.ctypes.data, int(divide))
    return tuple(int(v) for v in out)


def clip_quantise(cloud, origin, max_range, res):
    """int32 (N,5): valid, clipped, end voxel xyz."""
    lib = load()
    arr, n, stride = _cloud(cloud)
    rec = np.zeros((n, 5), np.int32)
    lib.vo_clip_quantise(arr.ctypes.data, n, stride, _d3(origin), float(max_range), float(res),
                         rec.ctypes.data)
    return rec


def clip_quantise_variant(cloud, origin, max_range, res, w2i_divide=False, unit_reciprocal=False):
    """As clip_quantise, under an arithmetic variant of the OpenVDB facts."""
    lib = load()
    arr, n, stride = _cloud(cloud)
    rec = np.zeros((n, 5), np.int32)
    lib.vo_clip_quantise_variant(arr.ctypes.data, n, stride, _d3(origin), float(max_range), float(res),
                                 int(w2i_divide), int(unit_reciprocal), rec.ctypes.data)
    return rec


MORPH_OPS = {"dilate": 0, "erode": 1, "close": 2, "open": 3}


def morphology(origins, masks, op, iterations, keep_leaves=False):
    """dilate / erode / close / open with the 26-neighbourhood (VDBMapping.hpp:1094-1147)
    of leaves (origins (n,3), OpenVDB-order masks (n,8)): (origins, masks) sorted by origin.
    keep_leaves: every input leaf and every leaf a dilation step reached stays, empty or not."""
    lib = load()
    o = np.ascontiguousarray(np.asarray(origins, np.int32).reshape(-1, 3))
    m = np.ascontiguousarray(np.asarray(masks, np.uint64).reshape(-1, 8))
    code = MORPH_OPS[op] | (16 if keep_leaves else 0)
    n = lib.vo_morphology(len(o), o.ctypes.data, m.ctypes.data, code, int(iterations), 0, None, None)
    oo = np.zeros((n, 3), np.int32)
    om = np.zeros((n, 8), np.uint64)
    lib.vo_morphology(len(o), o.ctypes.data, m.ctypes.data, code, int(iterations), n, oo.ctypes.data,
                      om.ctypes.data)
    return oo, om


def close_value_section(origins, values, masks, iterations):
    """morphologicalCloseMap of a value section (applyMapSectionGrid with smoothing,
    VDBMapping.hpp:1026-1029): (origins, values, masks) sorted by origin."""
    lib = load()
    o = np.ascontiguousarray(np.asarray(origins, np.int32).reshape(-1, 3))
    v = np.ascontiguousarray(np.asarray(values, np.float32).reshape(-1, 512))
    m = np.ascontiguousarray(np.asarray(masks, np.uint64).reshape(-1, 8))
    n = lib.vo_close_value_section(len(o), o.ctypes.data, v.ctypes.data, m.ctypes.data, int(iterations), 0, None,
                                   None, None)
    oo = np.zeros((n, 3), np.int32)
    ov = np.zeros((n, 512), np.float32)
    om = np.zeros((n, 8), np.uint64)
    lib.vo_close_value_section(len(o), o.ctypes.data, v.ctypes.data, m.ctypes.data, int(iterations), n,
                               oo.ctypes.data, ov.ctypes.data, om.ctypes.data)
    return oo, ov, om


def bench_replicas(res, cfg, scans, origins, threads):
    """Wall seconds for `threads` independent CPU maps each inserting all scans."""
    lib = load()
    scans = np.ascontiguousarray(np.asarray(scans, np.float32))
    s, n, k = scans.shape
    origins = np.ascontiguousarray(np.asarray(origins, np.float64))
    cfg7 = (C.c_double * 7)(cfg.max_range, float(cfg.fast_mode), cfg.accumulation_period, cfg.prob_hit,
                            cfg.prob_miss, cfg.prob_thres_min, cfg.prob_thres_max)
    st = (C.c_uint64 * 5)()
    sec = lib.vo_bench_replicas(float(res), cfg7, scans.ctypes.data, s, n, k,
                                origins.ctypes.data_as(C.POINTER(C.c_double)), int(threads), st)
    return sec, dict(zip(STAT_KEYS, list(st)))
