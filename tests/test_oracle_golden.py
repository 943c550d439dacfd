"""Pins the CPU oracle to the reference's own known answers
(test/testGWRBasic.cpp, absolute tolerance 1e-8) before anything trusts it."""
import math

import numpy as np
import pytest

import oracle as O


def _check_diag(diag, exp, tol):
    for key in ("AIC", "AICc", "RSquare", "RSquareAdjust"):
        assert abs(diag[key] - exp[key]) <= tol, (key, diag[key], exp[key])


def test_adaptive_gaussian_bw36(londonhp):
    e = londonhp["expected"]["adaptive_gaussian_bw36"]
    r = O.gwr_fit(londonhp["x"], londonhp["y"], londonhp["coords"], bandwidth=36, adaptive=True,
                  kernel=O.GAUSSIAN)
    _check_diag(r["diagnostic"], e, londonhp["tol"])


def test_fixed_gaussian_bw5000(londonhp):
    e = londonhp["expected"]["fixed_gaussian_bw5000"]
    r = O.gwr_fit(londonhp["x"], londonhp["y"], londonhp["coords"], bandwidth=5000, adaptive=False,
                  kernel=O.GAUSSIAN)
    _check_diag(r["diagnostic"], e, londonhp["tol"])


def test_adaptive_cv_search_selects_67(londonhp):
    e = londonhp["expected"]["adaptive_gaussian_cv_search"]
    r = O.gwr_fit(londonhp["x"], londonhp["y"], londonhp["coords"], adaptive=True, kernel=O.GAUSSIAN,
                  autoselect_bandwidth=True, criterion=O.CV)
    assert r["bandwidth"] == e["selected_bandwidth"]


def test_variable_selection_criteria(londonhp):
    e = londonhp["expected"]["variable_selection_aic"]
    r = O.gwr_fit(londonhp["x"], londonhp["y"], londonhp["coords"], bandwidth=36, adaptive=True,
                  kernel=O.GAUSSIAN, autoselect_vars=True, var_threshold=e["threshold"])
    got = r["var_criterion_list"]
    assert [v for v, _ in got] == [v for v, _ in e["criterion_list"]]
    for (_, a), (_, b) in zip(got, e["criterion_list"]):
        assert abs(a - b) <= londonhp["tol"]
    assert r["selected_vars"] == e["selected"]


def test_cv_search_after_variable_selection(londonhp):
    e = londonhp["expected"]["cv_search_with_variable_selection"]
    r = O.gwr_fit(londonhp["x"], londonhp["y"], londonhp["coords"], bandwidth=36, adaptive=True,
                  kernel=O.GAUSSIAN, autoselect_vars=True, var_threshold=e["threshold"],
                  autoselect_bandwidth=True, criterion=O.CV)
    assert r["selected_vars"] == e["selected"]
    assert r["bandwidth"] == e["selected_bandwidth"]
    _check_diag(r["diagnostic"], e, londonhp["tol"])


def test_adaptive_threshold_interpolates():
    """BandwidthWeight.cpp:41-49: fixbw = s[b0-1] + (s[b0]-s[b0-1]) * frac(b)."""
    d = np.array([5.0, 1.0, 3.0, 2.0, 4.0])
    assert O.adaptive_threshold(d, 2) == 2.0
    assert O.adaptive_threshold(d, 2.25) == 2.0 + (3.0 - 2.0) * 0.25
    assert O.adaptive_threshold(d, 5) == 5.0          # dn >= 1: (bw/n) * max
    assert O.adaptive_threshold(d, 7.5) == 1.5 * 5.0
    with pytest.raises(IndexError):
        O.adaptive_threshold(d, 0.5)


def test_kernels_match_formulas():
    """BandwidthWeight.h:68-121 evaluated by hand."""
    d = np.array([0.0, 0.5, 1.0, 2.0])
    bw = 1.0
    libm_exp = np.vectorize(math.exp)  # the reference's exp is libm's, not numpy's SIMD exp
    np.testing.assert_array_equal(O.weight(d, bw, False, O.GAUSSIAN), libm_exp(d * d / (-2.0 * (bw * bw))))
    np.testing.assert_array_equal(O.weight(d, bw, False, O.EXPONENTIAL), libm_exp(-d / bw))
    t = 1.0 - d * d / (bw * bw)
    np.testing.assert_array_equal(O.weight(d, bw, False, O.BISQUARE), (d < bw) * (t * t))
    t3 = 1.0 - d * d * d / (bw * bw * bw)
    np.testing.assert_array_equal(O.weight(d, bw, False, O.TRICUBE), (d < bw) * (t3 * t3 * t3))
    np.testing.assert_array_equal(O.weight(d, bw, False, O.BOXCAR), (d < bw) * 1.0)


def test_portable_great_circle_close_to_libm():
    """The engine's portable sin/cos/atan reproduce the libm SpGcdist
    (CRSDistance.cpp:15-69) to a few ulp over the config-2 domain and globally."""
    rng = np.random.default_rng(7)
    worst = 0.0
    exact = 0
    N = 20000
    for k in range(N):
        if k % 2:
            lon1, lon2 = rng.uniform(-10, 30, 2)
            lat1, lat2 = rng.uniform(35, 60, 2)
        else:
            lon1, lon2 = rng.uniform(-180, 180, 2)
            lat1, lat2 = rng.uniform(-89, 89, 2)
        a = O.gcdist(lon1, lon2, lat1, lat2, O.GC_LIBM)
        b = O.gcdist(lon1, lon2, lat1, lat2, O.GC_PORTABLE)
        exact += a == b
        worst = max(worst, abs(a - b) / a)
    assert worst < 1e-14, worst
    assert exact > N // 4


def test_great_circle_edge_cases():
    assert O.gcdist(10, 10, 45, 45) == 0.0
    assert O.gcdist(180, -180, 10, 10) == 0.0      # |lon1|+|lon2| == 360 branch
    near = O.gcdist(10.0, 10.0 + 1e-6, 45.0, 45.0 + 1e-6)
    assert 0.0 < near < 1e-3
    np.testing.assert_allclose(near, O.gcdist(10.0, 10.0 + 1e-6, 45.0, 45.0 + 1e-6, O.GC_LIBM), rtol=1e-9)
