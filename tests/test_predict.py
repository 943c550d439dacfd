"""GWRBasic::predict (GWRBasic.cpp:130-191).

CPU: the oracle's predict restatement at the data points themselves equals
its fit (a prediction at a data point is that point's local regression).
GPU: the engine's FP64 predict against the oracle at 1e-10 relative (planar
and geographic, adaptive and fixed kernels, fractional adaptive bandwidths),
at the data points against the engine's own fit at 1e-12, and through the
GWRBasic facade."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

from libgwmodel_gb300 import datasets  # noqa: E402


def problem(n, p, geo, seed):
    return datasets._plain_problem(np.random.default_rng(seed), n, p, geo, "predict")


def locations(pb, nr, seed):
    rng = np.random.default_rng(seed)
    lo, hi = pb.coords.min(0), pb.coords.max(0)
    return np.asfortranarray(rng.uniform(lo, hi, (nr, 2)))


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_oracle_predict_at_data_points_is_the_fit():
    pb = problem(300, 4, False, 1)
    prob = O.Problem(pb.x, pb.y, pb.coords, geographic=False)
    b_fit = prob.fit_core(40, True, 2, store_s=False)[0]
    b_pred = prob.predict(pb.coords, 40, True, 2)
    assert rel(b_pred, b_fit) <= 1e-14


CASES = [("planar adaptive bisquare", False, True, 2, 45.0), ("planar adaptive fractional", False, True, 2, 60.5),
         ("planar fixed gaussian", False, False, 0, 12.0), ("geographic adaptive bisquare", True, True, 2, 50.0),
         ("geographic fixed tricube", True, False, 3, 900.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("name,geo,adaptive,kernel,bw", CASES)
def test_engine_predict_matches_oracle(name, geo, adaptive, kernel, bw):
    from libgwmodel_gb300 import Engine
    pb = problem(1500, 5, geo, 3)
    loc = locations(pb, 400, 4)
    prob = O.Problem(pb.x, pb.y, pb.coords, geographic=geo)
    want = prob.predict(loc, bw, adaptive, kernel)
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, geo)
    got = e.predict(loc, bw, adaptive, kernel)
    for k in range(pb.p):
        assert rel(got[:, k], want[:, k]) <= 1e-10, (name, k)


@pytest.mark.gpu
def test_predict_at_data_points_equals_fit():
    from libgwmodel_gb300 import Engine
    pb = problem(2000, 6, True, 5)
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, True)
    b_fit = e.fit(70, True, 2, store_s=False)[0]
    b_pred = e.predict(pb.coords, 70, True, 2)
    assert rel(b_pred, b_fit) <= 1e-12


@pytest.mark.gpu
def test_facade_predict():
    from libgwmodel_gb300 import BandwidthWeight, CRSDistance, GWRBasic, SpatialWeight
    pb = problem(1200, 4, False, 6)
    loc = locations(pb, 250, 7)
    alg = GWRBasic()
    alg.setCoords(pb.coords)
    alg.setDependentVariable(pb.y)
    alg.setIndependentVariables(pb.x)
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(55, True, BandwidthWeight.Bisquare), CRSDistance(False)))
    got = alg.predict(loc)
    assert got.shape == (250, 4)
    want = O.Problem(pb.x, pb.y, pb.coords, geographic=False).predict(loc, 55, True, 2)
    assert rel(got, want) <= 1e-10
