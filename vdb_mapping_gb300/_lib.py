"""ctypes binding of the C ABI in include/vdb_gb300.h (libvdb_gb300.so).

The library is the only compute path: if it is missing this module raises,
there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

VDBG_POINTS_DEVICE = 1
VDBG_NOALLOC_MAX_POINTS = 262144
VDBG_NOALLOC_SCRATCH_BYTES = 28 << 20

STATUS = {
    0: "VDBG_OK",
    1: "VDBG_ERR_NOT_CONFIGURED",
    2: "VDBG_ERR_UNKNOWN_SOURCE",
    3: "VDBG_ERR_BAD_RANGE",
    4: "VDBG_ERR_BAD_PROBABILITY",
    5: "VDBG_ERR_DUPLICATE_SOURCE",
    6: "VDBG_ERR_INVALID_ARGUMENT",
    7: "VDBG_ERR_OUT_OF_MEMORY",
    8: "VDBG_ERR_COORD_RANGE",
    9: "VDBG_ERR_CUDA",
    10: "VDBG_ERR_TIMEOUT",
    11: "VDBG_ERR_BUFFER_TOO_SMALL",
    12: "VDBG_ERR_SIZE_LIMIT",
    13: "VDBG_ERR_BUSY",
}
STATUS_CODE = {v: k for k, v in STATUS.items()}


class vdbg_config(C.Structure):
    _fields_ = [
        ("max_range", C.c_double),
        ("fast_mode", C.c_int32),
        ("reserved0", C.c_int32),
        ("accumulation_period", C.c_double),
        ("prob_hit", C.c_double),
        ("prob_miss", C.c_double),
        ("prob_thres_min", C.c_double),
        ("prob_thres_max", C.c_double),
    ]


class vdbg_options(C.Structure):
    _fields_ = [
        ("initial_leaf_capacity", C.c_int64),
        ("max_device_bytes", C.c_int64),
        ("device", C.c_int32),
        ("initial_block_capacity", C.c_int32),
    ]


class vdbg_scan_stats(C.Structure):
    _fields_ = [
        ("rays", C.c_uint64),
        ("visits", C.c_uint64),
        ("hits", C.c_uint64),
        ("updates", C.c_uint64),
        ("new_leaves", C.c_uint64),
        ("touched_leaves", C.c_uint64),
        ("skipped_nonfinite", C.c_uint64),
        ("device_ms", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class vdbg_timings(C.Structure):
    _fields_ = [
        ("prep_ms", C.c_double),
        ("dda_ms", C.c_double),
        ("sweep_ms", C.c_double),
        ("total_ms", C.c_double),
        ("launches", C.c_uint64),
        ("launches_total", C.c_uint64),
        ("retries", C.c_uint64),
        ("apply_ms", C.c_double),
        ("runs", C.c_uint64),
        ("passes", C.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class vdbg_tuning(C.Structure):
    _fields_ = [
        ("rays_per_take", C.c_int32),
        ("apply_chunk_runs", C.c_int32),
        ("length_edges", C.c_int32 * 3),
        ("hash_load", C.c_float),
        ("dda_warps_per_sm", C.c_int32),
        ("sweep_kernel", C.c_int32),
    ]

    def as_dict(self):
        return {"rays_per_take": self.rays_per_take, "apply_chunk_runs": self.apply_chunk_runs,
                "length_edges": tuple(self.length_edges), "hash_load": round(float(self.hash_load), 4),
                "dda_warps_per_sm": self.dda_warps_per_sm, "sweep_kernel": self.sweep_kernel}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        t.rays_per_take = int(d["rays_per_take"])
        t.apply_chunk_runs = int(d["apply_chunk_runs"])
        for k in range(3):
            t.length_edges[k] = int(d["length_edges"][k])
        t.hash_load = float(d["hash_load"])
        t.dda_warps_per_sm = int(d.get("dda_warps_per_sm", 16))
        t.sweep_kernel = int(d.get("sweep_kernel", 0))
        return t


class vdbg_server_options(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_int64),
        ("max_batch_maps", C.c_int32),
        ("queue_capacity", C.c_int32),
    ]


class vdbg_server_result(C.Structure):
    _fields_ = [
        ("tag", C.c_uint64),
        ("map", C.c_int32),
        ("status", C.c_int32),
        ("points", C.c_int64),
        ("submit_ns", C.c_int64),
        ("start_ns", C.c_int64),
        ("done_ns", C.c_int64),
        ("batch_maps", C.c_int32),
        ("reserved0", C.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved0"}


class vdbg_server_stats(C.Structure):
    _fields_ = [
        ("requests_submitted", C.c_int64),
        ("requests_done", C.c_int64),
        ("rejected", C.c_int64),
        ("steps", C.c_int64),
        ("max_step_maps", C.c_int64),
        ("queued", C.c_int64),
        ("max_queued", C.c_int64),
        ("rays", C.c_uint64),
        ("updates", C.c_uint64),
        ("busy_ns", C.c_int64),
        ("device_bytes", C.c_int64),
        ("overlapped_steps", C.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class vdbg_pool_info(C.Structure):
    _fields_ = [
        ("leaf_capacity", C.c_int64),
        ("leaf_backed", C.c_int64),
        ("leaf_reserved", C.c_int64),
        ("leaves", C.c_int64),
        ("block_capacity", C.c_int64),
        ("blocks", C.c_int64),
        ("hash_entries", C.c_int64),
        ("grow_ahead", C.c_uint64),
        ("grow_sync", C.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# (name, restype, argtypes) of every exported entry point.
_P = C.c_void_p
_D3 = C.POINTER(C.c_double)
SIGNATURES = [
    ("vdbg_create", C.c_int, [C.c_double, C.POINTER(vdbg_options), C.POINTER(_P)]),
    ("vdbg_destroy", C.c_int, [_P]),
    ("vdbg_set_config", C.c_int, [_P, C.POINTER(vdbg_config)]),
    ("vdbg_get_log_odds", C.c_int, [_P, C.POINTER(C.c_float)]),
    ("vdbg_add_input_source", C.c_int, [_P, C.c_char_p, C.c_double, C.c_double]),
    ("vdbg_insert_point_cloud", C.c_int,
     [_P, _P, C.c_int64, C.c_int64, _D3, C.c_char_p, C.c_uint32, _P, C.POINTER(vdbg_scan_stats)]),
    ("vdbg_accumulate_update", C.c_int,
     [_P, _P, C.c_int64, C.c_int64, _D3, C.c_char_p, C.c_uint32, _P, C.POINTER(vdbg_scan_stats)]),
    ("vdbg_integrate_update", C.c_int, [_P, _P, C.POINTER(vdbg_scan_stats)]),
    ("vdbg_raycast_point_cloud", C.c_int,
     [_P, _P, C.c_int64, C.c_int64, _D3, C.c_double, C.c_char_p, C.c_uint32, _P,
      C.POINTER(vdbg_scan_stats)]),
    ("vdbg_update_map", C.c_int, [_P, C.c_char_p, _P, C.POINTER(vdbg_scan_stats)]),
    ("vdbg_reset_map", C.c_int, [_P]),
    ("vdbg_leaf_count", C.c_int, [_P, C.POINTER(C.c_int64)]),
    ("vdbg_export_leaves", C.c_int, [_P, C.c_int64, _P, _P, _P, C.POINTER(C.c_int64)]),
    ("vdbg_device_bytes", C.c_int, [_P, C.POINTER(C.c_int64)]),
    ("vdbg_get_timings", C.c_int, [_P, C.POINTER(vdbg_timings)]),
    ("vdbg_get_pool_info", C.c_int, [_P, C.POINTER(vdbg_pool_info)]),
    ("vdbg_ray_digests", C.c_int, [_P, _P, C.c_int64, C.c_int64, _D3, C.c_double, C.c_uint32, _P]),
    ("vdbg_map_digest", C.c_int, [_P, C.c_int, C.POINTER(C.c_uint64)]),
    ("vdbg_l2_atomic_rate", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("vdbg_insert_point_cloud_noalloc", C.c_int,
     [_P, _P, C.c_int64, C.c_int64, _D3, C.c_char_p, C.c_uint32, _P, C.POINTER(vdbg_scan_stats)]),
    ("vdbg_track_changes", C.c_int, [_P, C.c_int]),
    ("vdbg_export_changes", C.c_int, [_P, C.c_int, C.c_int64, _P, _P, _P, C.POINTER(C.c_int64)]),
    ("vdbg_set_tuning", C.c_int, [_P, C.POINTER(vdbg_tuning)]),
    ("vdbg_get_tuning", C.c_int, [_P, C.POINTER(vdbg_tuning)]),
    ("vdbg_create_batch", C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(vdbg_options), C.POINTER(_P)]),
    ("vdbg_batch_set_config", C.c_int, [_P, C.c_int, C.POINTER(vdbg_config)]),
    ("vdbg_batch_insert", C.c_int,
     [_P, _P, C.POINTER(C.c_int64), C.c_int64, C.POINTER(C.c_double), C.c_uint32, _P,
      C.POINTER(vdbg_scan_stats)]),
    ("vdbg_export_section", C.c_int, [_P, C.c_int, _P, _P, C.c_int, C.c_int64, _P, _P, _P, C.POINTER(C.c_int64)]),
    ("vdbg_apply_section_states", C.c_int, [_P, C.c_int, _P, _P, C.c_int64, _P, _P]),
    ("vdbg_apply_section_values", C.c_int, [_P, C.c_int, C.c_int64, _P, _P, _P]),
    ("vdbg_raytrace", C.c_int, [_P, C.c_int, C.c_int64, _P, _P, _P, _P, _P]),
    ("vdbg_add_artificial_walls", C.c_int, [_P, C.c_int64, _P, _P, C.c_double, C.c_double]),
    ("vdbg_restore_map_integrity", C.c_int, [_P]),
    ("vdbg_test_stall_leaf", C.c_int, [_P, C.c_int, C.c_int32, C.c_int32, C.c_int32]),
    ("vdbg_section_morphology", C.c_int, [_P, C.c_int, C.c_int, C.c_int64, _P, _P, C.c_int64, _P, _P,
                                          C.POINTER(C.c_int64)]),
    ("vdbg_batch_use_graph", C.c_int, [_P, C.c_int]),
    ("vdbg_graph_stats", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("vdbg_batch_leaf_count", C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    ("vdbg_batch_export_leaves", C.c_int, [_P, C.c_int, C.c_int64, _P, _P, _P, C.POINTER(C.c_int64)]),
    ("vdbg_server_create", C.c_int, [_P, C.POINTER(vdbg_server_options), C.POINTER(_P)]),
    ("vdbg_server_submit", C.c_int, [_P, C.c_int, _P, C.c_int64, C.c_int64, C.POINTER(C.c_double), C.c_uint64]),
    ("vdbg_server_poll", C.c_int, [_P, C.POINTER(vdbg_server_result), C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("vdbg_server_drain", C.c_int, [_P, C.c_int]),
    ("vdbg_server_get_stats", C.c_int, [_P, C.POINTER(vdbg_server_stats)]),
    ("vdbg_server_destroy", C.c_int, [_P]),
    ("vdbg_status_string", C.c_char_p, [C.c_int]),
]

_lib = None


def load(path: str | None = None):
    """Loads libvdb_gb300.so (building it first if absent) and binds it."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from .build import build_library
        build_library()
    if not os.path.exists(p):
        raise RuntimeError(f"libvdb_gb300.so not found at {p}; run vdb_mapping_gb300.build")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class VdbgError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        text = load().vdbg_status_string(status).decode()
        super().__init__(f"{where}: {STATUS.get(status, status)} ({text})")
