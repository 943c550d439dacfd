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


def _gc_pairs(n, seed):
    rng = np.random.default_rng(seed)
    half = n // 2
    lon = np.concatenate([rng.uniform(-10, 30, (half, 2)), rng.uniform(-180, 180, (n - half, 2))])
    lat = np.concatenate([rng.uniform(35, 60, (half, 2)), rng.uniform(-89, 89, (n - half, 2))])
    return lon, lat


def test_correctly_rounded_sin_cos_atan(gc_host):
    """gw_sincos_cr and gw_atan_cr return the correctly rounded double
    (checked against 160-bit arithmetic) over the arguments the great-circle
    formula takes: half-sums and half-differences of radians, and
    sqrt(S / C) from 0 to the far side of the globe."""
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 160
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-6.3, 6.3, 4000), rng.uniform(0.6, 0.9, 2000),
                        rng.uniform(-1, 1, 2000) * 10.0 ** rng.uniform(-12, 0, 2000)])
    s, c = gc_host.sincos(x)
    assert all(float(mp.sin(v)) == a for v, a in zip(x, s))
    assert all(float(mp.cos(v)) == a for v, a in zip(x, c))
    t = np.concatenate([rng.uniform(0, 2, 4000), 10.0 ** rng.uniform(-14, 14, 4000)])
    a = gc_host.atan(t)
    assert all(float(mp.atan(v)) == r for v, r in zip(t, a))


def test_great_circle_against_libm(gc_host):
    """The engine's SpGcdist (CRSDistance.cpp:15-69) with correctly rounded
    sin/cos/atan against the same formula with the platform libm.  glibc
    rounds a small fraction of sin/cos/atan results the other way, so the
    stated bar is: at most 2% of distances differ, each by at most 8 ulp
    (measured here: ~0.7% of pairs, <= 2 ulp)."""
    lon, lat = _gc_pairs(20000, 7)
    coords = np.column_stack([np.concatenate([lon[:, 0], lon[:, 1]]), np.concatenate([lat[:, 0], lat[:, 1]])])
    row = gc_host.rows(coords)
    n = len(lon)
    differ, worst = 0, 0
    for k in range(0, n, 40):
        d_cr = row(n + k)[:n]  # focus (lon2, lat2) against every data point (lon1, lat1)
        for j in range(k, min(k + 40, n)):
            ref = O.gcdist(lon[j, 0], lon[k, 1], lat[j, 0], lat[k, 1])
            if ref != d_cr[j]:
                differ += 1
                worst = max(worst, abs(int(np.float64(ref).view(np.int64)) - int(np.float64(d_cr[j]).view(np.int64))))
    assert differ <= 0.02 * n, differ
    assert worst <= 8, worst


@pytest.mark.parametrize("delta", [1e-1, 1e-3, 1e-5])
def test_great_circle_near_the_antipode(gc_host, delta):
    """Pairs within delta rad of each other's antipode, where the Lambert
    correction's 1/cos^2 terms grow: the correctly rounded form and libm stay
    within the bar of test_great_circle_against_libm, and the distances stay
    finite and near half the meridian circumference (the whole-sphere GPU test
    selects on such pairs)."""
    rng = np.random.default_rng(11)
    n = 600
    lon1 = rng.uniform(-180.0, 180.0, n)
    lat1 = np.degrees(np.arcsin(rng.uniform(-0.99, 0.99, n)))
    ang = rng.uniform(0.0, 2.0 * np.pi, n)
    lon2 = lon1 + 180.0 + np.degrees(delta * np.cos(ang) / np.cos(np.radians(lat1)))
    lon2 = (lon2 + 180.0) % 360.0 - 180.0
    lat2 = -lat1 + np.degrees(delta * np.sin(ang))
    row = gc_host.rows(np.column_stack([np.concatenate([lon1, lon2]), np.concatenate([lat1, lat2])]))
    cr = np.array([row(n + k)[k] for k in range(n)])
    libm = np.array([O.gcdist(lon1[k], lon2[k], lat1[k], lat2[k]) for k in range(n)])
    assert np.all(np.isfinite(cr)) and np.all(np.isfinite(libm))
    assert np.all((cr > 19000.0) & (cr < 20100.0)), (cr.min(), cr.max())
    ulp = np.abs(cr.view(np.int64) - libm.view(np.int64))
    assert (ulp > 0).sum() <= 0.02 * n and ulp.max() <= 8, (int((ulp > 0).sum()), int(ulp.max()))


def test_great_circle_edge_cases():
    assert O.gcdist(10, 10, 45, 45) == 0.0
    assert O.gcdist(180, -180, 10, 10) == 0.0      # |lon1|+|lon2| == 360 branch
    near = O.gcdist(10.0, 10.0 + 1e-6, 45.0, 45.0 + 1e-6)
    assert 0.0 < near < 1e-3
    np.testing.assert_allclose(near, 2 * 6378.137 * math.radians(1e-6) * 0.5 * math.sqrt(1 + math.cos(math.radians(45)) ** 2),
                               rtol=1e-2)
