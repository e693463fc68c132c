"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports
every entry point include/vdb_gb300.h declares (no GPU work is launched)."""
import ctypes as C
import os
import re
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "vdb_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(vdbg_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from vdb_mapping_gb300.build import build_library

    return build_library()


def test_header_declares_the_path():
    fns = declared_functions()
    for name in ["vdbg_create", "vdbg_destroy", "vdbg_set_config", "vdbg_add_input_source",
                 "vdbg_insert_point_cloud", "vdbg_accumulate_update", "vdbg_integrate_update",
                 "vdbg_raycast_point_cloud", "vdbg_update_map", "vdbg_reset_map", "vdbg_export_leaves"]:
        assert name in fns


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (vdbg_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_library_loads_and_binds(lib_path):
    from vdb_mapping_gb300 import _lib

    lib = _lib.load()
    for name, _, _ in _lib.SIGNATURES:
        assert hasattr(lib, name)
    # The Python binding covers every entry point of the header.
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_status_strings(lib_path):
    from vdb_mapping_gb300 import _lib

    lib = _lib.load()
    for code in _lib.STATUS:
        assert lib.vdbg_status_string(code)
    assert lib.vdbg_status_string(1).decode().startswith("Map not properly configured")


def test_struct_layouts_match_header():
    from vdb_mapping_gb300 import _lib

    assert C.sizeof(_lib.vdbg_config) == 56
    assert C.sizeof(_lib.vdbg_options) == 24
    assert C.sizeof(_lib.vdbg_scan_stats) == 64


STRUCTS = ("vdbg_config", "vdbg_options", "vdbg_scan_stats", "vdbg_timings", "vdbg_pool_info", "vdbg_tuning",
           "vdbg_server_options", "vdbg_server_result", "vdbg_server_stats")


def test_ctypes_mirrors_match_the_compiled_header(tmp_path):
    """Every struct of include/vdb_gb300.h, compiled by the C compiler: its
    size and every field's offset equal the ctypes mirror's."""
    from vdb_mapping_gb300 import _lib

    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "vdb_gb300.h"', "int main(void) {"]
    for name in STRUCTS:
        cls = getattr(_lib, name)
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layouts"
    include = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    res = subprocess.run(["gcc", "-std=c11", "-I", include, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            *key, value = line.split()
            got[tuple(key)] = int(value)
    for name in STRUCTS:
        cls = getattr(_lib, name)
        assert got[(name, "size")] == C.sizeof(cls), name
        for field, _ in cls._fields_:
            assert got[(name, field)] == getattr(cls, field).offset, (name, field)


def test_build_targets_sm_103a_only():
    from vdb_mapping_gb300 import build

    flags = " ".join(build.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert flags.count("-gencode") == 1
    assert "-fmad=false" in flags


def test_new_entry_points_reject_bad_arguments_before_device_work(lib_path):
    """Argument checks of the raytrace and morphology entry points run before
    any CUDA call, so they hold without a GPU."""
    from vdb_mapping_gb300 import _lib

    lib = _lib.load()
    bad = _lib.STATUS_CODE["VDBG_ERR_INVALID_ARGUMENT"]
    n = C.c_int64(7)
    d3 = (C.c_double * 3)()
    ok = (C.c_uint8 * 1)()
    # no map
    assert lib.vdbg_raytrace(None, -1, 1, d3, d3, d3, ok, d3) == bad
    assert lib.vdbg_section_morphology(None, 2, 1, 0, None, None, 0, None, None, C.byref(n)) == bad
    # unknown op, iterations out of range, missing outputs: checked before the map is used
    fake = C.c_void_p(1)
    assert lib.vdbg_section_morphology(fake, 4, 1, 0, None, None, 0, None, None, C.byref(n)) == bad
    assert lib.vdbg_section_morphology(fake, 2, 65, 0, None, None, 0, None, None, C.byref(n)) == bad
    assert lib.vdbg_section_morphology(fake, 2, 1, 1, None, None, 0, None, None, C.byref(n)) == bad
    assert lib.vdbg_section_morphology(fake, 2, 1, 0, None, None, 0, None, None, None) == bad
    o = (C.c_int32 * 3)(3, 0, 0)  # not a multiple of 8
    m = (C.c_uint64 * 8)()
    assert lib.vdbg_section_morphology(fake, 2, 1, 1, o, m, 0, None, None, C.byref(n)) == bad
    o = (C.c_int32 * 3)(1 << 21, 0, 0)  # beyond +-2^20
    assert lib.vdbg_section_morphology(fake, 2, 1, 1, o, m, 0, None, None, C.byref(n)) == \
        _lib.STATUS_CODE["VDBG_ERR_COORD_RANGE"]
