import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
ORACLE_DIR = os.path.join(REPO, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.load()
    return O


@pytest.fixture(scope="session")
def vdbg():
    """The CUDA library; a GPU test fails (not skips) when it cannot load."""
    if not gpu_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    import vdb_mapping_gb300 as V

    V.load()
    return V
