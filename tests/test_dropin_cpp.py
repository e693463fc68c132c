"""The reference-style C++ API (include/vdb_mapping/*.hpp) over the C ABI.

CPU: the reference's own tests/mapping.cpp (when the reference tree is on
this machine) and tests/cpp/dropin_test.cpp compile and link against the
drop-in headers and libvdb_gb300.so unchanged; the OpenVDB build of the
drop-in compiles against declarations of the third-party API it calls
(tests/cpp/third_party_api). GPU: dropin_test and openvdb_adapter_test run.
"""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("VDB_MAPPING_REFERENCE", "/root/reference")
OUT = os.path.join(REPO, "tests", "cpp", "_build")


def compile_against_dropin(src, exe, extra=()):
    from vdb_mapping_gb300.build import BUILD_DIR, build_library

    build_library()
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", *extra, "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(REPO, "oracle", "refshim"),  # only for the minimal gtest.h
           src, "-L", BUILD_DIR, "-lvdb_gb300", f"-Wl,-rpath,{BUILD_DIR}", "-o", os.path.join(OUT, exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return os.path.join(OUT, exe)


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "tests", "mapping.cpp")),
                    reason="reference tree not present on this machine")
def test_reference_unit_tests_compile_against_dropin():
    compile_against_dropin(os.path.join(REF, "tests", "mapping.cpp"), "reference_mapping_tests")


def test_dropin_test_compiles():
    compile_against_dropin(os.path.join(REPO, "tests", "cpp", "dropin_test.cpp"), "dropin_test")


# The OpenVDB build of the drop-in (VDBG_WITH_OPENVDB), against declarations of
# the OpenVDB / PCL / Eigen API surface it uses (the libraries are not installed).
OPENVDB_API = ("-DVDBG_WITH_OPENVDB", "-I", os.path.join(REPO, "tests", "cpp", "third_party_api"))


def test_openvdb_adapter_compiles():
    compile_against_dropin(os.path.join(REPO, "tests", "cpp", "openvdb_adapter_test.cpp"),
                           "openvdb_adapter_test", OPENVDB_API)


@pytest.mark.gpu
def test_openvdb_adapter_runs_on_gpu():
    src = os.path.join(REPO, "tests", "cpp", "openvdb_adapter_test.cpp")
    exe = compile_against_dropin(src, "openvdb_adapter_test", OPENVDB_API)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    n_cases = open(src).read().count("\nTEST(")
    assert n_cases >= 2
    assert f"{n_cases} tests, 0 failed" in res.stdout


@pytest.mark.gpu
def test_dropin_test_runs_on_gpu():
    exe = compile_against_dropin(os.path.join(REPO, "tests", "cpp", "dropin_test.cpp"), "dropin_test")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    n_cases = open(os.path.join(REPO, "tests", "cpp", "dropin_test.cpp")).read().count("\nTEST(")
    assert n_cases >= 6
    assert f"{n_cases} tests, 0 failed" in res.stdout
