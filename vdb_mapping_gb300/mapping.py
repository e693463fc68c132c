"""Python mirror of vdb_mapping's OccupancyVDBMapping over the C ABI.

Names, argument meaning and error behaviour follow the reference
(include/vdb_mapping/VDBMapping.hpp, include/vdb_mapping/OccupancyVDBMapping.hpp):
errors that the reference prints and swallows are printed and swallowed here
too (``insertPointCloud`` always returns True, VDBMapping.hpp:399-406);
everything else the library reports raises ``VdbgError``.

Point clouds are ``numpy`` arrays of shape (N, 3) or (N, 4) float32 in host
memory (a pcl::PointXYZ cloud is (N, 4)), or CUDA ``torch`` tensors of the same
shapes, which are read in place on the device.
"""
from __future__ import annotations

import ctypes as C
import sys
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import VdbgError


@dataclass
class Config:
    """vdb_mapping::Config (OccupancyVDBMapping.hpp:38-44) + BaseConfig (VDBMapping.hpp:64-71)."""

    max_range: float = 0.0
    fast_mode: bool = False
    accumulation_period: float = 0.0
    prob_hit: float = 0.0
    prob_miss: float = 0.0
    prob_thres_min: float = 0.0
    prob_thres_max: float = 0.0
    map_directory_path: str = ""


def _cloud_args(cloud):
    """(pointer, n, stride_bytes, flags, keepalive) for a numpy array or CUDA tensor."""
    if hasattr(cloud, "is_cuda") and cloud.is_cuda:
        import torch

        if cloud.dtype != torch.float32 or cloud.dim() != 2 or cloud.shape[1] < 3:
            raise ValueError("CUDA cloud must be a float32 tensor of shape (N, 3+)")
        if cloud.stride(1) != 1:
            cloud = cloud.contiguous()
        return cloud.data_ptr(), cloud.shape[0], cloud.stride(0) * 4, _lib.VDBG_POINTS_DEVICE, cloud
    if hasattr(cloud, "numpy") and not isinstance(cloud, np.ndarray):
        cloud = cloud.numpy()
    arr = np.asarray(cloud)
    if arr.dtype != np.float32:
        arr = arr.astype(np.float32)
    if arr.ndim != 2 or arr.shape[1] < 3:
        raise ValueError("cloud must have shape (N, 3) or (N, 4)")
    if arr.strides[1] != 4 or arr.strides[0] % 4:
        arr = np.ascontiguousarray(arr)
    return arr.ctypes.data, arr.shape[0], arr.strides[0], 0, arr


def _origin(origin):
    o = (C.c_double * 3)(*[float(v) for v in origin])
    return o


def _export_changes(lib, h, map_index, check):
    """(origins (L,3) int32, active (L,8) uint64, value (L,8) uint64) of the
    last integration's change set."""
    n = C.c_int64()
    cap = 1024
    while True:
        origins = np.zeros((cap, 3), np.int32)
        active = np.zeros((cap, 8), np.uint64)
        value = np.zeros((cap, 8), np.uint64)
        s = lib.vdbg_export_changes(h, int(map_index), cap, origins.ctypes.data, active.ctypes.data,
                                    value.ctypes.data, C.byref(n))
        if s == _lib.STATUS_CODE["VDBG_ERR_BUFFER_TOO_SMALL"]:
            cap = n.value
            continue
        check(s, "vdbg_export_changes")
        k = n.value
        return origins[:k], active[:k], value[:k]


class Grid:
    """Export of the map (VDBMapping::getGrid, VDBMapping.hpp:799).

    Holds the leaves sorted by origin: ``origins`` (L,3) int32, ``values``
    (L,512) float32 log-odds in OpenVDB leaf order, ``masks`` (L,8) uint64
    active masks. ``getAccessor()`` gives OpenVDB-style point queries. A grid
    obtained from a mapping re-exports itself when the map has changed since,
    so an accessor taken before an insertion sees its result (as an OpenVDB
    accessor on the live grid does).
    """

    def __init__(self, origins, values, masks, owner=None, version=-1):
        self._set(origins, values, masks)
        self._owner = owner
        self._version = version

    def _set(self, origins, values, masks):
        self.origins = origins
        self.values = values
        self.masks = masks
        self._index = {tuple(o): i for i, o in enumerate(origins.tolist())}

    def _sync(self):
        if self._owner is not None and self._owner._version != self._version:
            o, v, m = self._owner._export()
            self._set(o, v, m)
            self._version = self._owner._version

    def leafCount(self) -> int:
        self._sync()
        return len(self.origins)

    def activeVoxelCount(self) -> int:
        self._sync()
        return int(sum(bin(int(w)).count("1") for w in self.masks.ravel()))

    def getAccessor(self):
        return _Accessor(self)

    def _lookup(self, xyz):
        self._sync()
        x, y, z = (int(c) for c in xyz)
        i = self._index.get((x & ~7, y & ~7, z & ~7))
        off = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7)
        return i, off

    def getValue(self, xyz) -> float:
        i, off = self._lookup(xyz)
        return 0.0 if i is None else float(self.values[i, off])

    def isValueOn(self, xyz) -> bool:
        i, off = self._lookup(xyz)
        if i is None:
            return False
        return bool((int(self.masks[i, off >> 6]) >> (off & 63)) & 1)


class _Accessor:
    def __init__(self, grid: Grid):
        self._g = grid

    def getValue(self, xyz) -> float:
        return self._g.getValue(xyz)

    def isValueOn(self, xyz) -> bool:
        return self._g.isValueOn(xyz)


def createIndexBoundingBox(min_boundary, max_boundary, map_to_reference_tf, resolution):
    """createIndexBoundingBox (VDBMapping.hpp:811-870): the eight corners of the
    world box as float points, transformed by the 4x4 matrix (each coordinate
    computed in double as row . (x, y, z, 1) and stored as float, as
    pcl::transformPointCloud does with a double matrix), their float min/max,
    then worldToIndex (w * (1/res)) and Coord::floor. Returns (lo, hi) int32."""
    lo_w = np.asarray(min_boundary, np.float64)
    hi_w = np.asarray(max_boundary, np.float64)
    tf = np.asarray(map_to_reference_tf, np.float64).reshape(4, 4)
    corners = []
    for cx in (lo_w[0], hi_w[0]):
        for cy in (lo_w[1], hi_w[1]):
            for cz in (lo_w[2], hi_w[2]):
                p = [float(np.float32(cx)), float(np.float32(cy)), float(np.float32(cz))]
                q = []
                for r in range(3):
                    acc = tf[r, 0] * p[0]
                    acc = acc + tf[r, 1] * p[1]
                    acc = acc + tf[r, 2] * p[2]
                    acc = acc + tf[r, 3]
                    q.append(np.float32(acc))
                corners.append(q)
    c = np.array(corners, np.float32)
    inv = 1.0 / float(resolution)
    lo = np.floor(c.min(axis=0).astype(np.float64) * inv).astype(np.int32)
    hi = np.floor(c.max(axis=0).astype(np.float64) * inv).astype(np.int32)
    return lo, hi


def _section_export(lib, h, map_index, lo, hi, full, check):
    lo = np.ascontiguousarray(lo, np.int32)
    hi = np.ascontiguousarray(hi, np.int32)
    n = C.c_int64()
    cap = 0
    while True:
        origins = np.zeros((cap, 3), np.int32)
        values = np.zeros((cap, 512), np.float32)
        masks = np.zeros((cap, 8), np.uint64)
        s = lib.vdbg_export_section(h, int(map_index), lo.ctypes.data, hi.ctypes.data, 1 if full else 0, cap,
                                    origins.ctypes.data, values.ctypes.data, masks.ctypes.data, C.byref(n))
        if s == _lib.STATUS_CODE["VDBG_ERR_BUFFER_TOO_SMALL"]:
            cap = n.value
            continue
        check(s, "vdbg_export_section")
        k = n.value
        return origins[:k], values[:k], masks[:k]


def _section_states(lib, h, map_index, lo, hi, origins, masks, check):
    lo = np.ascontiguousarray(lo, np.int32)
    hi = np.ascontiguousarray(hi, np.int32)
    o = np.ascontiguousarray(origins, np.int32).reshape(-1, 3)
    mk = np.ascontiguousarray(masks, np.uint64).reshape(-1, 8)
    check(lib.vdbg_apply_section_states(h, int(map_index), lo.ctypes.data, hi.ctypes.data, len(o), o.ctypes.data,
                                        mk.ctypes.data), "vdbg_apply_section_states")


def _section_values(lib, h, map_index, origins, values, masks, check):
    o = np.ascontiguousarray(origins, np.int32).reshape(-1, 3)
    v = np.ascontiguousarray(values, np.float32).reshape(-1, 512)
    mk = np.ascontiguousarray(masks, np.uint64).reshape(-1, 8)
    check(lib.vdbg_apply_section_values(h, int(map_index), len(o), o.ctypes.data, v.ctypes.data, mk.ctypes.data),
          "vdbg_apply_section_values")


MORPH_OPS = {"dilate": 0, "erode": 1, "close": 2, "open": 3}


MORPH_KEEP_LEAVES = 16  # VDBG_MORPH_KEEP_LEAVES


def _morphology(lib, h, origins, masks, op, iterations, check, keep_leaves=False):
    o = np.ascontiguousarray(np.asarray(origins, np.int32).reshape(-1, 3))
    mk = np.ascontiguousarray(np.asarray(masks, np.uint64).reshape(-1, 8))
    code = MORPH_OPS[op] | (MORPH_KEEP_LEAVES if keep_leaves else 0)
    n = C.c_int64()
    cap = 0
    while True:
        oo = np.zeros((cap, 3), np.int32)
        om = np.zeros((cap, 8), np.uint64)
        s = lib.vdbg_section_morphology(h, code, int(iterations), len(o), o.ctypes.data, mk.ctypes.data, cap,
                                        oo.ctypes.data, om.ctypes.data, C.byref(n))
        if s == _lib.STATUS_CODE["VDBG_ERR_BUFFER_TOO_SMALL"]:
            cap = n.value
            continue
        check(s, "vdbg_section_morphology")
        return oo[: n.value], om[: n.value]


def _close_value_section(lib, h, origins, values, masks, iterations, check):
    """morphologicalCloseMap of a value section (VDBMapping.hpp:1026-1029, 1094-1099):
    the active voxels closed with every leaf kept; the leaves the dilation adds hold 0."""
    o = np.asarray(origins, np.int32).reshape(-1, 3)
    v = np.asarray(values, np.float32).reshape(-1, 512)
    ro, rm = _morphology(lib, h, o, masks, "close", iterations, check, keep_leaves=True)
    rv = np.zeros((len(ro), 512), np.float32)
    where = {tuple(int(c) for c in org): i for i, org in enumerate(o)}
    for j, org in enumerate(ro):
        i = where.get(tuple(int(c) for c in org))
        if i is not None:
            rv[j] = v[i]
    return ro, rv, rm


def _raytrace(lib, h, map_index, origins, directions, max_lengths, check):
    o = np.ascontiguousarray(np.asarray(origins, np.float64).reshape(-1, 3))
    d = np.ascontiguousarray(np.asarray(directions, np.float64).reshape(-1, 3))
    n = o.shape[0]
    if d.shape[0] != n:
        raise ValueError("origins and directions differ in length")
    ln = np.ascontiguousarray(np.broadcast_to(np.asarray(max_lengths, np.float64), (n,)))
    ok = np.zeros(n, np.uint8)
    ends = np.zeros((n, 3), np.float64)
    check(lib.vdbg_raytrace(h, int(map_index), n, o.ctypes.data, d.ctypes.data, ln.ctypes.data, ok.ctypes.data,
                            ends.ctypes.data), "vdbg_raytrace")
    return ok.astype(bool), ends


class OccupancyVDBMapping:
    """vdb_mapping::OccupancyVDBMapping (OccupancyVDBMapping.hpp:46-200) on the GPU."""

    def __init__(self, resolution: float, initial_leaf_capacity: int = 0, max_device_bytes: int = 0,
                 device: int | None = None, initial_block_capacity: int = 0):
        self._lib = _lib.load()
        opts = _lib.vdbg_options()
        opts.initial_leaf_capacity = int(initial_leaf_capacity)
        opts.initial_block_capacity = int(initial_block_capacity)
        opts.max_device_bytes = int(max_device_bytes)
        if device is None:
            try:
                import torch

                device = torch.cuda.current_device() if torch.cuda.is_available() else 0
            except Exception:  # pragma: no cover - torch is plumbing only
                device = 0
        opts.device = int(device)
        h = C.c_void_p()
        s = self._lib.vdbg_create(float(resolution), C.byref(opts), C.byref(h))
        if s != 0:
            raise VdbgError(s, "vdbg_create")
        self._h = h
        self.resolution = float(resolution)
        self._version = 0
        self._grid = None
        self.last_stats = None

    # -- lifetime -----------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.vdbg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, s, where, swallow=()):
        if s == 0:
            return True
        if s in swallow:
            return False
        raise VdbgError(s, where)

    # -- configuration (OccupancyVDBMapping.hpp:59-89, VDBMapping.hpp:1352-1375) ----
    def setConfig(self, config: Config) -> None:
        c = _lib.vdbg_config()
        c.max_range = config.max_range
        c.fast_mode = 1 if config.fast_mode else 0
        c.accumulation_period = config.accumulation_period
        c.prob_hit = config.prob_hit
        c.prob_miss = config.prob_miss
        c.prob_thres_min = config.prob_thres_min
        c.prob_thres_max = config.prob_thres_max
        s = self._lib.vdbg_set_config(self._h, C.byref(c))
        if s == _lib.STATUS_CODE["VDBG_ERR_BAD_RANGE"]:
            print(f"Max range of {config.max_range} invalid. Range cannot be negative.", file=sys.stderr)
        elif s == _lib.STATUS_CODE["VDBG_ERR_BAD_PROBABILITY"]:
            if config.prob_miss > 0.5:
                print(f"Probability for a miss should be below 0.5 but is {config.prob_miss}", file=sys.stderr)
            else:
                print(f"Probability for a hit should be above 0.5 but is {config.prob_hit}", file=sys.stderr)
        else:
            self._check(s, "vdbg_set_config")

    def logOdds(self):
        out = (C.c_float * 6)()
        self._check(self._lib.vdbg_get_log_odds(self._h, out), "vdbg_get_log_odds")
        keys = ("hit", "miss", "thres_min", "thres_max", "max", "min")
        return dict(zip(keys, list(out)))

    def addInputSource(self, source_id: str, max_range: float, max_rate: float) -> None:
        self._check(self._lib.vdbg_add_input_source(self._h, source_id.encode(), float(max_range),
                                                    float(max_rate)), "vdbg_add_input_source")

    # -- the hot path -------------------------------------------------------------
    def _cloud_call(self, fn, cloud, origin, *extra, stream=None):
        ptr, n, stride, flags, keep = _cloud_args(cloud)
        st = _lib.vdbg_scan_stats()
        s = fn(self._h, C.c_void_p(ptr), n, stride, _origin(origin), *extra, flags,
               C.c_void_p(stream) if stream else None, C.byref(st))
        del keep
        self.last_stats = st.as_dict()
        self._version += 1
        return s

    def insertPointCloud(self, cloud, origin, source_id: str, stream=None) -> bool:
        """VDBMapping.hpp:399-406; always True, like the reference."""
        s = self._cloud_call(self._lib.vdbg_insert_point_cloud, cloud, origin, source_id.encode(),
                             stream=stream)
        if s == _lib.STATUS_CODE["VDBG_ERR_UNKNOWN_SOURCE"]:
            print(f"Tried to accumulate update for {source_id}. Source not available")
        elif s == _lib.STATUS_CODE["VDBG_ERR_NOT_CONFIGURED"]:
            print("Map not properly configured. Did you call setConfig method?", file=sys.stderr)
        else:
            self._check(s, "vdbg_insert_point_cloud")
        return True

    def accumulateUpdate(self, cloud, origin, source_id: str, stream=None) -> None:
        """VDBMapping.hpp:316-346."""
        s = self._cloud_call(self._lib.vdbg_accumulate_update, cloud, origin, source_id.encode(),
                             stream=stream)
        if s == _lib.STATUS_CODE["VDBG_ERR_UNKNOWN_SOURCE"]:
            print(f"Tried to accumulate update for {source_id}. Source not available")
        elif s == _lib.STATUS_CODE["VDBG_ERR_NOT_CONFIGURED"]:
            print("Map not properly configured. Did you call setConfig method?", file=sys.stderr)
        else:
            self._check(s, "vdbg_accumulate_update")

    def integrateUpdate(self, stream=None) -> None:
        """VDBMapping.hpp:375-387."""
        st = _lib.vdbg_scan_stats()
        s = self._lib.vdbg_integrate_update(self._h, C.c_void_p(stream) if stream else None, C.byref(st))
        self.last_stats = st.as_dict()
        self._version += 1
        self._check(s, "vdbg_integrate_update")

    def raycastPointCloud(self, cloud, origin, raycast_range: float, source_id: str, stream=None) -> bool:
        """VDBMapping.hpp:466-539 into the update grid of `source_id`."""
        s = self._cloud_call(self._lib.vdbg_raycast_point_cloud, cloud, origin, float(raycast_range),
                             source_id.encode(), stream=stream)
        if s == _lib.STATUS_CODE["VDBG_ERR_NOT_CONFIGURED"]:
            print("Map not properly configured. Did you call setConfig method?", file=sys.stderr)
            return False
        self._check(s, "vdbg_raycast_point_cloud")
        return True

    def updateMap(self, source_id: str, stream=None) -> None:
        """VDBMapping.hpp:731-792 for one source's update grid."""
        st = _lib.vdbg_scan_stats()
        s = self._lib.vdbg_update_map(self._h, source_id.encode(), C.c_void_p(stream) if stream else None,
                                      C.byref(st))
        self.last_stats = st.as_dict()
        self._version += 1
        self._check(s, "vdbg_update_map")

    def resetMap(self) -> None:
        """VDBMapping.hpp:174-186."""
        self._check(self._lib.vdbg_reset_map(self._h), "vdbg_reset_map")
        self._version += 1
        self._grid = None

    # -- export -------------------------------------------------------------------
    def leafCount(self) -> int:
        n = C.c_int64()
        self._check(self._lib.vdbg_leaf_count(self._h, C.byref(n)), "vdbg_leaf_count")
        return n.value

    def timings(self) -> dict:
        """Per-phase device times and launch counts of the last call."""
        t = _lib.vdbg_timings()
        self._check(self._lib.vdbg_get_timings(self._h, C.byref(t)), "vdbg_get_timings")
        return t.as_dict()

    def deviceBytes(self) -> int:
        n = C.c_int64()
        self._check(self._lib.vdbg_device_bytes(self._h, C.byref(n)), "vdbg_device_bytes")
        return n.value

    def poolInfo(self) -> dict:
        """Leaf and block pool sizes and how often they grew (ahead / on demand)."""
        p = _lib.vdbg_pool_info()
        self._check(self._lib.vdbg_get_pool_info(self._h, C.byref(p)), "vdbg_get_pool_info")
        return p.as_dict()

    def rayDigests(self, cloud, origin, raycast_range: float) -> np.ndarray:
        """uint64 (N, 2): per point, castRayIntoGrid's visit count with the
        clipped and valid flags, and a hash chain over the visited voxels
        (vdbg_ray_digests). The map is not changed."""
        ptr, n, stride, flags, keep = _cloud_args(cloud)
        out = np.zeros((n, 2), np.uint64)
        s = self._lib.vdbg_ray_digests(self._h, C.c_void_p(ptr), n, stride, _origin(origin), float(raycast_range),
                                       flags, out.ctypes.data)
        del keep
        self._check(s, "vdbg_ray_digests")
        return out

    def mapDigest(self) -> tuple:
        """(leaves, voxels, leaf sum, voxel sum) of the map (vdbg_map_digest)."""
        out = (C.c_uint64 * 4)()
        self._check(self._lib.vdbg_map_digest(self._h, 0, out), "vdbg_map_digest")
        return tuple(int(v) for v in out)

    def setTuning(self, tuning: dict) -> None:
        """Kernel launch/layout parameters (speed only; results never change)."""
        t = _lib.vdbg_tuning.from_dict(tuning)
        self._check(self._lib.vdbg_set_tuning(self._h, C.byref(t)), "vdbg_set_tuning")

    def tuning(self) -> dict:
        t = _lib.vdbg_tuning()
        self._check(self._lib.vdbg_get_tuning(self._h, C.byref(t)), "vdbg_get_tuning")
        return t.as_dict()

    def trackChanges(self, enable: bool = True) -> None:
        """Keep the change set of each integration (updateMap's change grid,
        VDBMapping.hpp:731-792)."""
        self._check(self._lib.vdbg_track_changes(self._h, 1 if enable else 0), "vdbg_track_changes")

    def getMapSection(self, lo, hi, full: bool = False):
        """getMapSectionGrid over the index box [lo, hi] (see createIndexBoundingBox):
        (origins, values, masks) sorted by origin; full=False gives value 1 at the
        active voxels (getMapSectionUpdateGrid reads the same as bool)."""
        return _section_export(self._lib, self._h, -1, lo, hi, full, self._check)

    def applyMapSectionStates(self, lo, hi, origins, masks, smooth: bool = False, iterations: int = 2) -> None:
        """applyMapSectionUpdateGrid with the section's box [lo, hi]; smooth closes
        the section's active voxels first (VDBMapping.hpp:1062-1065)."""
        if smooth:
            origins, masks = self.sectionMorphology(origins, masks, "close", iterations)
        _section_states(self._lib, self._h, -1, lo, hi, origins, masks, self._check)

    def addArtificialWall(self, start, end, negative_height: float, positive_height: float) -> None:
        """addArtificialWall (VDBMapping.hpp:1210-1236): the wall's voxels are set
        active after every update of the map (x, y, z of start and end are used)."""
        st = np.ascontiguousarray(np.asarray(start, np.float64)[:3])
        en = np.ascontiguousarray(np.asarray(end, np.float64)[:3])
        self._check(self._lib.vdbg_add_artificial_walls(self._h, 1, st.ctypes.data, en.ctypes.data,
                                                        float(negative_height), float(positive_height)),
                    "vdbg_add_artificial_walls")

    def addArtificialPolygon(self, polygon, negative_height: float, positive_height: float) -> None:
        """addArtificialPolygon (VDBMapping.hpp:1198-1207): walls between consecutive corners, closed."""
        pts = np.asarray(polygon, np.float64).reshape(len(polygon), -1)[:, :3]
        if len(pts) == 0:
            return
        st = np.ascontiguousarray(pts)
        en = np.ascontiguousarray(np.roll(pts, -1, axis=0))
        self._check(self._lib.vdbg_add_artificial_walls(self._h, len(pts), st.ctypes.data, en.ctypes.data,
                                                        float(negative_height), float(positive_height)),
                    "vdbg_add_artificial_walls")

    def addArtificialAreas(self, areas, negative_height: float, positive_height: float) -> None:
        """addArtificialAreas (VDBMapping.hpp:1175-1189): restoreMapIntegrity, then every polygon."""
        self.restoreMapIntegrity()
        for poly in areas:
            self.addArtificialPolygon(poly, negative_height, positive_height)

    def restoreMapIntegrity(self) -> None:
        """restoreMapIntegrity (VDBMapping.hpp:1153-1166)."""
        self._check(self._lib.vdbg_restore_map_integrity(self._h), "vdbg_restore_map_integrity")
        self._version += 1

    def sectionMorphology(self, origins, masks, op: str = "close", iterations: int = 2, keep_leaves: bool = False):
        """morphologicalDilateMap / ErodeMap / CloseMap / OpenMap (VDBMapping.hpp:1094-1147)
        of a section's active voxels on the GPU: op in dilate, erode, close, open.
        Returns (origins, masks) of the leaves with active voxels, sorted by origin;
        keep_leaves: every input leaf and every leaf a dilation reached, empty or not."""
        return _morphology(self._lib, self._h, origins, masks, op, iterations, self._check, keep_leaves)

    def applyMapSectionValues(self, origins, values, masks, smooth: bool = False, iterations: int = 2) -> None:
        """applyMapSectionGrid; smooth closes the section first (VDBMapping.hpp:1026-1029)."""
        if smooth:
            origins, values, masks = _close_value_section(self._lib, self._h, origins, values, masks, iterations,
                                                          self._check)
        _section_values(self._lib, self._h, -1, origins, values, masks, self._check)

    def raytrace(self, origins, directions, max_lengths):
        """raytrace (VDBMapping.hpp:675-721) for n rays (world origins and
        directions (n, 3), lengths (n,) or one length): (successes bool (n,),
        end points (n, 3)). One ray: raytrace([o], [d], length)."""
        return _raytrace(self._lib, self._h, -1, origins, directions, max_lengths, self._check)

    def exportChanges(self):
        """Change set of the last integration: (origins, active, value) per leaf
        with a flip, sorted by origin; `value` marks voxels flipped on by a hit."""
        return _export_changes(self._lib, self._h, -1, self._check)

    def _export(self):
        n = C.c_int64()
        cap = self.leafCount()
        while True:
            origins = np.zeros((cap, 3), np.int32)
            values = np.zeros((cap, 512), np.float32)
            masks = np.zeros((cap, 8), np.uint64)
            s = self._lib.vdbg_export_leaves(self._h, cap, origins.ctypes.data, values.ctypes.data,
                                             masks.ctypes.data, C.byref(n))
            if s == _lib.STATUS_CODE["VDBG_ERR_BUFFER_TOO_SMALL"]:
                cap = n.value
                continue
            self._check(s, "vdbg_export_leaves")
            k = n.value
            return origins[:k], values[:k], masks[:k]

    def exportLeaves(self):
        """(origins, values, masks) sorted by leaf origin."""
        return self._export()

    def getGrid(self) -> Grid:
        if self._grid is None:
            self._grid = Grid(np.zeros((0, 3), np.int32), np.zeros((0, 512), np.float32),
                              np.zeros((0, 8), np.uint64), owner=self, version=-1)
        return self._grid


def _config_struct(config: Config):
    c = _lib.vdbg_config()
    c.max_range = config.max_range
    c.fast_mode = 1 if config.fast_mode else 0
    c.accumulation_period = config.accumulation_period
    c.prob_hit = config.prob_hit
    c.prob_miss = config.prob_miss
    c.prob_thres_min = config.prob_thres_min
    c.prob_thres_max = config.prob_thres_max
    return c


class MapBatch:
    """Independent occupancy maps in one device pool, one scan per map per call.

    No counterpart in the reference, which holds one OccupancyVDBMapping per
    map: ``insert`` is ``insertPointCloud`` (VDBMapping.hpp:399-406) for every
    map at once, with each map's own resolution and setConfig
    (OccupancyVDBMapping.hpp:59-89). Each map's result equals inserting its
    scan alone into its own map.
    """

    def __init__(self, resolutions, initial_leaf_capacity: int = 0, max_device_bytes: int = 0,
                 device: int | None = None, initial_block_capacity: int = 0):
        self._lib = _lib.load()
        self.resolutions = [float(r) for r in resolutions]
        opts = _lib.vdbg_options()
        opts.initial_leaf_capacity = int(initial_leaf_capacity)
        opts.initial_block_capacity = int(initial_block_capacity)
        opts.max_device_bytes = int(max_device_bytes)
        if device is None:
            try:
                import torch

                device = torch.cuda.current_device() if torch.cuda.is_available() else 0
            except Exception:  # pragma: no cover - torch is plumbing only
                device = 0
        opts.device = int(device)
        res = (C.c_double * len(self.resolutions))(*self.resolutions)
        h = C.c_void_p()
        s = self._lib.vdbg_create_batch(len(self.resolutions), res, C.byref(opts), C.byref(h))
        if s != 0:
            raise VdbgError(s, "vdbg_create_batch")
        self._h = h
        self.last_stats = None

    def __len__(self):
        return len(self.resolutions)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.vdbg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, s, where):
        if s != 0:
            raise VdbgError(s, where)

    def setConfig(self, map_index: int, config: Config) -> None:
        c = _config_struct(config)
        self._check(self._lib.vdbg_batch_set_config(self._h, int(map_index), C.byref(c)), "vdbg_batch_set_config")

    def insert(self, clouds, origins, stream=None) -> dict:
        """One scan per map: ``clouds[i]`` ((N,3)/(N,4) float32 host array, or None)
        from ``origins[i]``. Returns the summed scan statistics."""
        n_maps = len(self.resolutions)
        if len(clouds) != n_maps or len(origins) != n_maps:
            raise ValueError("one cloud and one origin per map")
        parts, counts = [], []
        for c in clouds:
            if c is None:
                counts.append(0)
                continue
            a = np.asarray(c, dtype=np.float32)
            if a.ndim != 2 or a.shape[1] < 3:
                raise ValueError("cloud must have shape (N, 3) or (N, 4)")
            if a.shape[1] != 4:
                a = np.concatenate([a[:, :3], np.zeros((a.shape[0], 1), np.float32)], axis=1)
            parts.append(np.ascontiguousarray(a))
            counts.append(a.shape[0])
        pts = np.concatenate(parts) if parts else np.zeros((0, 4), np.float32)
        return self.insert_packed(pts, counts, origins, stream=stream)

    def insert_packed(self, pts, counts, origins, stream=None) -> dict:
        """``pts``: (sum(counts), 4) float32 host array (or CUDA tensor) holding
        the maps' scans back to back in map order."""
        ptr, n, stride, flags, keep = _cloud_args(pts)
        cnt = (C.c_int64 * len(counts))(*[int(c) for c in counts])
        if n != sum(int(c) for c in counts):
            raise ValueError("counts do not add up to the number of points")
        org = (C.c_double * (3 * len(origins)))(*[float(v) for o in origins for v in o])
        st = _lib.vdbg_scan_stats()
        s = self._lib.vdbg_batch_insert(self._h, C.c_void_p(ptr), cnt, stride, org, flags,
                                        C.c_void_p(stream) if stream else None, C.byref(st))
        del keep
        self.last_stats = st.as_dict()
        self._check(s, "vdbg_batch_insert")
        return self.last_stats

    def leafCount(self, map_index: int) -> int:
        n = C.c_int64()
        self._check(self._lib.vdbg_batch_leaf_count(self._h, int(map_index), C.byref(n)), "vdbg_batch_leaf_count")
        return n.value

    def setTuning(self, tuning: dict) -> None:
        """Kernel launch/layout parameters (speed only; results never change)."""
        t = _lib.vdbg_tuning.from_dict(tuning)
        self._check(self._lib.vdbg_set_tuning(self._h, C.byref(t)), "vdbg_set_tuning")

    def tuning(self) -> dict:
        t = _lib.vdbg_tuning()
        self._check(self._lib.vdbg_get_tuning(self._h, C.byref(t)), "vdbg_get_tuning")
        return t.as_dict()

    def trackChanges(self, enable: bool = True) -> None:
        self._check(self._lib.vdbg_track_changes(self._h, 1 if enable else 0), "vdbg_track_changes")

    def useGraph(self, enable: bool = True) -> None:
        """Replay each batched step as one captured CUDA graph (default on;
        results are the same either way)."""
        self._check(self._lib.vdbg_batch_use_graph(self._h, 1 if enable else 0), "vdbg_batch_use_graph")

    def graphStats(self) -> dict:
        c, r = C.c_uint64(), C.c_uint64()
        self._check(self._lib.vdbg_graph_stats(self._h, C.byref(c), C.byref(r)), "vdbg_graph_stats")
        return {"captures": c.value, "replays": r.value}

    def getMapSection(self, map_index: int, lo, hi, full: bool = False):
        return _section_export(self._lib, self._h, map_index, lo, hi, full, self._check)

    def applyMapSectionStates(self, map_index: int, lo, hi, origins, masks, smooth: bool = False,
                              iterations: int = 2) -> None:
        if smooth:
            origins, masks = self.sectionMorphology(origins, masks, "close", iterations)
        _section_states(self._lib, self._h, map_index, lo, hi, origins, masks, self._check)

    def sectionMorphology(self, origins, masks, op: str = "close", iterations: int = 2, keep_leaves: bool = False):
        """See OccupancyVDBMapping.sectionMorphology."""
        return _morphology(self._lib, self._h, origins, masks, op, iterations, self._check, keep_leaves)

    def applyMapSectionValues(self, map_index: int, origins, values, masks, smooth: bool = False,
                              iterations: int = 2) -> None:
        if smooth:
            origins, values, masks = _close_value_section(self._lib, self._h, origins, values, masks, iterations,
                                                          self._check)
        _section_values(self._lib, self._h, map_index, origins, values, masks, self._check)

    def raytrace(self, map_index: int, origins, directions, max_lengths):
        """raytrace on one map of the batch (see OccupancyVDBMapping.raytrace)."""
        return _raytrace(self._lib, self._h, map_index, origins, directions, max_lengths, self._check)

    def exportChanges(self, map_index: int):
        """Change set of the last batched insert for one map."""
        return _export_changes(self._lib, self._h, map_index, self._check)

    def exportLeaves(self, map_index: int):
        """(origins, values, masks) of one map, sorted by leaf origin."""
        n = C.c_int64()
        cap = self.leafCount(map_index)
        while True:
            origins = np.zeros((cap, 3), np.int32)
            values = np.zeros((cap, 512), np.float32)
            masks = np.zeros((cap, 8), np.uint64)
            s = self._lib.vdbg_batch_export_leaves(self._h, int(map_index), cap, origins.ctypes.data,
                                                   values.ctypes.data, masks.ctypes.data, C.byref(n))
            if s == _lib.STATUS_CODE["VDBG_ERR_BUFFER_TOO_SMALL"]:
                cap = n.value
                continue
            self._check(s, "vdbg_batch_export_leaves")
            k = n.value
            return origins[:k], values[:k], masks[:k]

    def timings(self) -> dict:
        t = _lib.vdbg_timings()
        self._check(self._lib.vdbg_get_timings(self._h, C.byref(t)), "vdbg_get_timings")
        return t.as_dict()

    def deviceBytes(self) -> int:
        n = C.c_int64()
        self._check(self._lib.vdbg_device_bytes(self._h, C.byref(n)), "vdbg_device_bytes")
        return n.value

    def poolInfo(self) -> dict:
        """Leaf and block pool sizes and how often they grew (ahead / on demand)."""
        p = _lib.vdbg_pool_info()
        self._check(self._lib.vdbg_get_pool_info(self._h, C.byref(p)), "vdbg_get_pool_info")
        return p.as_dict()

    def mapDigest(self, map_index: int) -> tuple:
        """(leaves, voxels, leaf sum, voxel sum) of one map (vdbg_map_digest)."""
        out = (C.c_uint64 * 4)()
        self._check(self._lib.vdbg_map_digest(self._h, int(map_index), out), "vdbg_map_digest")
        return tuple(int(v) for v in out)


class MapServer:
    """Continuous-batching request loop over a ``MapBatch`` (vdbg_server_*).

    ``submit`` queues one scan for one map and returns at once; a native
    worker thread inserts the oldest queued scan of every map in one batched
    call per step, admitting scans against ``memory_budget_bytes``; ``poll``
    returns completed requests with their steady-clock submit/start/done
    times in ns. While the server runs only it may use the batch.
    """

    def __init__(self, batch: "MapBatch", memory_budget_bytes: int = 0, max_batch_maps: int = 0,
                 queue_capacity: int = 0):
        self._lib = _lib.load()
        self.batch = batch
        opts = _lib.vdbg_server_options()
        opts.memory_budget_bytes = int(memory_budget_bytes)
        opts.max_batch_maps = int(max_batch_maps)
        opts.queue_capacity = int(queue_capacity)
        h = C.c_void_p()
        s = self._lib.vdbg_server_create(batch._h, C.byref(opts), C.byref(h))
        if s != 0:
            raise VdbgError(s, "vdbg_server_create")
        self._h = h

    def submit(self, map_index: int, cloud, origin, tag: int = 0) -> int:
        """Queues a host cloud ((N,3)/(N,4) float32); returns the status
        (VDBG_ERR_BUSY when the queue is full)."""
        ptr, n, stride, flags, keep = _cloud_args(cloud)
        if flags:
            raise ValueError("the server stages host clouds")
        s = self._lib.vdbg_server_submit(self._h, int(map_index), C.c_void_p(ptr), n, stride, _origin(origin),
                                         int(tag))
        del keep
        if s not in (0, _lib.STATUS_CODE["VDBG_ERR_BUSY"]):
            raise VdbgError(s, "vdbg_server_submit")
        return s

    def poll(self, capacity: int = 256, wait_ms: int = 0):
        buf = (_lib.vdbg_server_result * capacity)()
        n = C.c_int()
        s = self._lib.vdbg_server_poll(self._h, buf, capacity, int(wait_ms), C.byref(n))
        if s != 0:
            raise VdbgError(s, "vdbg_server_poll")
        return [buf[i].as_dict() for i in range(n.value)]

    def drain(self, wait_ms: int = 60000) -> None:
        s = self._lib.vdbg_server_drain(self._h, int(wait_ms))
        if s != 0:
            raise VdbgError(s, "vdbg_server_drain")

    def stats(self) -> dict:
        st = _lib.vdbg_server_stats()
        s = self._lib.vdbg_server_get_stats(self._h, C.byref(st))
        if s != 0:
            raise VdbgError(s, "vdbg_server_get_stats")
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.vdbg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
