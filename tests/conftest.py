import ctypes
import json
import os
import subprocess
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


def mgwr_kwargs(case, p):
    """Oracle / engine keyword arguments of one MGWR known-answer case of the golden
    fixture (per-variable lists of length p)."""
    init = {"Null": 0, "Initial": 1, "Specified": 2}[case["init"]]
    approach = {"CV": 0, "AIC": 1}[case["approach"]]
    return dict(bw0=[case["bw0"]] * p, adaptive=[int(case["adaptive"])] * p, kernel=[2] * p,
                init_type=[init] * p, approach=[approach] * p,
                centered=[int(c) for c in case["centered"]],
                select_threshold=[case["select_threshold"]] * p, retry_times=case["retry_times"],
                criterion_type={"CVR": 0, "dCVR": 1}[case["criterion"]],
                lower=case.get("lower"), upper=case.get("upper"), hat_matrix=case["hat_matrix"])


@pytest.fixture(scope="session")
def londonhp_mgwr():
    """The londonhp100 fixture as test/testGWRMultiscale.cpp:31-32 uses it:
    y = PURCHASE, X = [1, FLOORSZ, PROF], with that file's known answers."""
    with open(os.path.join(ROOT, "tests", "golden", "londonhp100.json")) as f:
        g = json.load(f)
    coords = np.array(g["coords"], dtype=np.float64)
    data = np.array(g["data"], dtype=np.float64)
    y = data[:, 0].copy()
    x = np.column_stack([np.ones(len(y)), data[:, 1], data[:, 3]])
    return {"coords": coords, "x": x, "y": y, "cases": g["mgwr"], "tol": g["mgwr_tolerance_abs"]}


class GcHost:
    """The engine's great-circle arithmetic (gw_arith.h) built for the host by
    tests/arith/gc_host.c: correctly rounded sin/cos/atan and exact distance rows."""

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        self._dp = ctypes.POINTER(ctypes.c_double)

    def _p(self, a):
        return a.ctypes.data_as(self._dp)

    def sincos(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        s, c = np.empty_like(x), np.empty_like(x)
        self.lib.gc_sincos_cr(self._p(x), self._p(s), self._p(c), len(x))
        return s, c

    def atan(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        a = np.empty_like(x)
        self.lib.gc_atan_cr(self._p(x), self._p(a), len(x))
        return a

    def rows(self, coords):
        """Distance rows (focus i against every point) for geographic coords."""
        lon = np.ascontiguousarray(coords[:, 0], dtype=np.float64)
        lat = np.ascontiguousarray(coords[:, 1], dtype=np.float64)
        n = len(lon)

        def row(i):
            out = np.empty(n)
            self.lib.gc_row_cr(self._p(lon), self._p(lat), n, int(i), self._p(out))
            return out
        return row


@pytest.fixture(scope="session")
def gc_host(tmp_path_factory):
    src = os.path.join(ROOT, "tests", "arith", "gc_host.c")
    out = str(tmp_path_factory.mktemp("gc_host") / "libgc_host.so")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", out, src, "-lm"])
    return GcHost(out)
