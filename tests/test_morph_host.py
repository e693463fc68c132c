"""The leaf-mask morphology of the section kernels
(vdb_mapping_gb300/csrc/morph.cuh), compiled for the host and driven the way
the kernels drive it, against the oracle's voxel-set restatement of OpenVDB's
dilateActiveValues / erodeActiveValues with the 26-neighbourhood: dilate,
erode, close and open on seeded random sections, bit for bit."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_host_morphology_matches_oracle():
    src = os.path.join(HERE, "cpp", "morph_host_test.cpp")
    out_dir = os.path.join(HERE, "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "morph_host_test")
    res = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-o", exe, src],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout[-3000:]
    assert run.stdout.strip().splitlines()[-1].startswith("ok ")
