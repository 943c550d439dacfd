import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def londonhp():
    """The londonhp100 fixture: y = PURCHASE, X = [1, FLOORSZ, UNEMPLOY, PROF]
    (test/testGWRBasic.cpp:27-28)."""
    with open(os.path.join(ROOT, "tests", "golden", "londonhp100.json")) as f:
        g = json.load(f)
    coords = np.array(g["coords"], dtype=np.float64)
    data = np.array(g["data"], dtype=np.float64)
    y = data[:, 0].copy()
    x = np.column_stack([np.ones(len(y)), data[:, 1:4]])
    return {"coords": coords, "x": x, "y": y, "expected": g["expected"], "tol": g["tolerance_abs"]}
