"""Reading and replaying the golden fixtures in tests/golden/*.npz.

A case holds the inputs of a short insertion sequence (resolution, config,
scans of pcl-layout points, origins) and the expected map as its leaves:
``origins`` (L,3) int32 sorted by (x, y, z), ``values`` (L,512) float32,
``masks`` (L,8) uint64. The fixtures were written by tests/golden/make_golden.py
from the oracle (whose own pins are tests/test_oracle.py).
"""
import numpy as np

from vdb_mapping_gb300.mapping import Config


def load_case(path):
    z = np.load(path)
    case = {k: z[k] for k in z.files}
    c = case["config"]
    case["cfg"] = Config(max_range=float(c[0]), fast_mode=bool(c[1]), accumulation_period=float(c[2]),
                         prob_hit=float(c[3]), prob_miss=float(c[4]), prob_thres_min=float(c[5]),
                         prob_thres_max=float(c[6]))
    case["res"] = float(case["resolution"])
    return case


def replay(m, case):
    m.setConfig(case["cfg"])
    m.addInputSource("golden", case["cfg"].max_range, 0)
    for pts, o in zip(case["scans"], case["scan_origins"]):
        m.insertPointCloud(pts, o, "golden")
    return m.exportLeaves()


def run_oracle_case(oracle, case):
    return replay(oracle.OracleMap(case["res"]), case)
