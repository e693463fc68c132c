"""The intersector traversal of the fast-mode and raytrace kernels
(vdb_mapping_gb300/csrc/hdda.cuh), compiled for the host, against the
oracle's separate restatement of OpenVDB's VolumeRayIntersector
(oracle/vdb_oracle.hpp): clipped rays, first spans, all spans, raytrace
results and fast-mode marks, bit for bit, on seeded random maps."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_host_traversal_matches_oracle():
    src = os.path.join(HERE, "cpp", "hdda_host_test.cpp")
    out_dir = os.path.join(HERE, "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "hdda_host_test")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-o", exe, src]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout[-3000:]
    assert run.stdout.strip().splitlines()[-1].startswith("ok ")
