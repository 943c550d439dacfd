"""Pins the oracle's GWRMultiscale restatement to the reference's known answers
(test/testGWRMultiscale.cpp: bandwidths to 0.1 or exactly, diagnostics to 1e-6)."""
import numpy as np
import pytest

import oracle as O
from conftest import mgwr_kwargs

CASES = ["fixed_null_cv_hat", "adaptive_initial_aic_hat_dcvr", "adaptive_null_cv_nohat",
         "adaptive_initial_cv_hat_cvr", "adaptive_null_cv_hat_cvr_bounds"]


@pytest.mark.parametrize("name", CASES)
def test_mgwr_known_answers(londonhp_mgwr, name):
    g = londonhp_mgwr
    case = g["cases"][name]
    pb = O.Problem(g["x"], g["y"], g["coords"], geographic=False)
    r = pb.mgwr(**mgwr_kwargs(case, pb.p))
    bws = r["bandwidths"]
    for got, want in zip(bws, case["bandwidths"]):
        if case["bandwidth_tol"] == 0.0:
            assert got == want, (bws, case["bandwidths"])
        else:
            assert abs(got - want) <= case["bandwidth_tol"], (bws, case["bandwidths"])
    for key in ("AICc", "RSquare", "RSquareAdjust"):
        if key in case:
            assert abs(r["diagnostic"][key] - case[key]) <= g["tol"], (key, r["diagnostic"][key], case[key])


def test_mgwr_single_variable_reduces_to_gwr(londonhp_mgwr):
    """With one column and its bandwidth fixed, back-fitting converges in one pass to
    the basic GWR fit at that bandwidth (GWRMultiscale.cpp fits the sole variable
    against the whole response)."""
    g = londonhp_mgwr
    x = np.ones((len(g["y"]), 1))
    pb = O.Problem(x, g["y"], g["coords"], geographic=False)
    r = pb.mgwr(bw0=[40], adaptive=[1], kernel=[2], init_type=[2], approach=[0], centered=[0],
                select_threshold=[1e-5], hat_matrix=True)
    ref = O.gwr_fit(x, g["y"], g["coords"], bandwidth=40, adaptive=True, kernel=O.BISQUARE)
    np.testing.assert_allclose(r["betas"], ref["betas"], rtol=1e-9, atol=1e-6)
