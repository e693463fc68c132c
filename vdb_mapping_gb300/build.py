"""Build recipe for the CUDA library (libvdb_gb300.so) and the CPU oracle.

The library is compiled in-tree with nvcc for sm_103a only; nothing is
installed. ``build()`` is what ``__graft_entry__.build()`` calls.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libvdb_gb300.so")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    # The log-odds update and the DDA are restated operation by operation;
    # no contraction into FMA anywhere (device or host).
    "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-shared",
]


def _sources():
    return [os.path.join(CSRC, "vdb_gb300.cu")]


def _deps():
    out = []
    for d in (CSRC, INCLUDE_DIR):
        for name in os.listdir(d):
            full = os.path.join(d, name)
            if os.path.isfile(full):
                out.append(full)
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and not _stale(LIB_PATH, _deps()):
        return LIB_PATH
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, *NVCC_FLAGS, "-I", INCLUDE_DIR, "-I", CSRC, *_sources(), "-o", LIB_PATH + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("nvcc failed building libvdb_gb300.so")
    if verbose:
        sys.stderr.write(res.stderr)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def build_oracle() -> None:
    """CPU oracle (test infrastructure): oracle/_build/liboracle.so."""
    res = subprocess.run(["make", "-s", "-C", os.path.join(REPO_DIR, "oracle"), "all"],
                         capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("building the oracle failed")


def build_reference_tests() -> bool:
    """The reference's own tests/mapping.cpp compiled against the oracle
    (outputs in oracle/_ref/), where the reference tree is present: the one
    the environment names (VDB_MAPPING_REFERENCE), else the oracle recipe's
    default location. Elsewhere nothing is built."""
    cmd = ["make", "-s", "-C", os.path.join(REPO_DIR, "oracle"), "ref-if-present"]
    ref = os.environ.get("VDB_MAPPING_REFERENCE")
    if ref:
        cmd.append(f"REF={ref}")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("building the reference tests against the oracle failed")
    return True


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, verbose), ex.submit(build_oracle), ex.submit(build_reference_tests)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB_PATH)
