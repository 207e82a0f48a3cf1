import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    if "x" not in d:  # lattice fixtures store no inputs: regenerate them exactly
        from petrbf_gb300 import workloads as W
        p = W.lamb_oseen_lattice_1e4()
        d["x"], d["y"] = p.x, p.y
    return d


@pytest.fixture(scope="session")
def golden():
    return load_golden
