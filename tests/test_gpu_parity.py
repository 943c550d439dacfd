"""GPU engine against the CPU oracle on the same seeded inputs.

Tolerances (FP64 drop-in): adaptive thresholds and the selected bandwidth
bit-exact; beta relative error <= 1e-10 (against the column's largest
|beta|); AICc and CV within 1e-9 relative; tr(S), tr(S^T S), qDiag, S and
betasSE within 1e-9 relative.

Geographic thresholds: see parity_util (bit-exact to the engine's correctly
rounded distances, libm's within the stated bar, identical neighbour sets)."""
import numpy as np
import pytest

import oracle as O
from parity_util import GEO_THR_ULP, check_geo_thresholds, col_rel, geo_rows as rows_of, rel, ulps
from libgwmodel_gb300 import BandwidthWeight, CRSDistance, Engine, GWRBasic, SpatialWeight, datasets

pytestmark = pytest.mark.gpu

KERNELS = [O.GAUSSIAN, O.EXPONENTIAL, O.BISQUARE, O.TRICUBE, O.BOXCAR]


@pytest.fixture(scope="module")
def planar():
    return datasets.config0(n=1500, seed=11)


@pytest.fixture(scope="module")
def geo():
    return datasets.config2(n=2000, seed=12, k=16)


@pytest.fixture(scope="module")
def geo_rows(geo, gc_host):
    """Distance rows of `geo`: (libm oracle, engine arithmetic on the host)."""
    return rows_of(geo.coords, range(geo.n), gc_host)


@pytest.fixture(scope="module")
def ties():
    """Coordinates on a coarse grid: many exactly equal distances."""
    rng = np.random.default_rng(13)
    n = 900
    coords = rng.integers(0, 12, (n, 2)).astype(np.float64)
    x = np.column_stack([np.ones(n), rng.standard_normal((n, 2))])
    y = x @ np.array([1.0, -2.0, 0.5]) + rng.normal(0, 0.3, n)
    return x, y, coords


def engine_for(x, y, coords, geographic=False):
    e = Engine(0)
    e.set_data(x, y, coords, geographic)
    return e


def oracle_thresholds(pb, bw):
    return np.array([O.adaptive_threshold(pb.distance_row(i), bw) for i in range(pb.n)])


@pytest.mark.parametrize("bw", [20, 37, 37.25, 400, 1499, 1500, 2250.5])
def test_adaptive_thresholds_bit_exact_planar(planar, bw):
    e = engine_for(planar.x, planar.y, planar.coords)
    pb = O.Problem(planar.x, planar.y, planar.coords)
    got = e.thresholds(bw)
    want = oracle_thresholds(pb, bw)
    assert np.array_equal(got, want), np.flatnonzero(got != want)[:10]


@pytest.mark.parametrize("bw", [20, 141, 350.5, 1351, 1999])
def test_adaptive_thresholds_geographic(geo, geo_rows, bw):
    e = engine_for(geo.x, geo.y, geo.coords, True)
    check_geo_thresholds(e.thresholds(bw), *geo_rows, bw)


@pytest.mark.parametrize("bw", [5, 33, 200, 450.5])
def test_adaptive_thresholds_with_ties(ties, bw):
    x, y, c = ties
    e = engine_for(x, y, c)
    pb = O.Problem(x, y, c)
    assert np.array_equal(e.thresholds(bw), oracle_thresholds(pb, bw))


def test_max_distance(planar, geo, geo_rows):
    e = engine_for(planar.x, planar.y, planar.coords)
    assert e.max_distance() == O.Problem(planar.x, planar.y, planar.coords).max_distance()
    g = engine_for(geo.x, geo.y, geo.coords, True)
    got = g.max_distance()
    assert got == max(d.max() for d in geo_rows[1])
    assert ulps(got, O.Problem(geo.x, geo.y, geo.coords, geographic=True).max_distance()) <= GEO_THR_ULP


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("criterion", [O.AIC, O.CV])
@pytest.mark.parametrize("adaptive", [True, False])
def test_criterion_planar(planar, kernel, criterion, adaptive):
    bw = 150 if adaptive else 12.0
    e = engine_for(planar.x, planar.y, planar.coords)
    pb = O.Problem(planar.x, planar.y, planar.coords)
    got = e.criterion(bw, adaptive, kernel, criterion)
    want, _ = pb.criterion(bw, adaptive, kernel, criterion)
    assert abs(got - want) <= 1e-9 * abs(want), (got, want)


@pytest.mark.parametrize("criterion", [O.AIC, O.CV])
def test_criterion_geographic(geo, criterion):
    e = engine_for(geo.x, geo.y, geo.coords, True)
    pb = O.Problem(geo.x, geo.y, geo.coords, geographic=True)
    for bw in (60, 301):
        got = e.criterion(bw, True, O.BISQUARE, criterion)
        want, _ = pb.criterion(bw, True, O.BISQUARE, criterion)
        assert abs(got - want) <= 1e-9 * abs(want), (bw, got, want)


@pytest.mark.parametrize("kernel,adaptive,bw", [(O.BISQUARE, True, 120), (O.GAUSSIAN, False, 9.0),
                                                (O.TRICUBE, True, 64.5)])
def test_fit_outputs(planar, kernel, adaptive, bw):
    n = 700
    x, y, c = planar.x[:n], planar.y[:n], planar.coords[:n]
    e = engine_for(x, y, c)
    pb = O.Problem(x, y, c)
    b, se, shat, q, S = e.fit(bw, adaptive, kernel, True)
    rb, rse, rshat, rq, rS = pb.fit_core(bw, adaptive, kernel, True)
    assert col_rel(b, rb) <= 1e-10
    assert col_rel(se, rse) <= 1e-9
    assert rel(shat, rshat) <= 1e-9
    assert rel(q, rq) <= 1e-9
    assert rel(S, rS) <= 1e-9
    # S is not stored: the reference keeps the last location's row
    _, _, _, q1, S1 = e.fit(bw, adaptive, kernel, False)
    assert S1.shape == (1, n) and rel(S1[0], rS[n - 1]) <= 1e-9
    assert rel(q1, rq) <= 1e-9


def test_global_criterion_matches_oracle(planar):
    e = engine_for(planar.x, planar.y, planar.coords)
    pb = O.Problem(planar.x, planar.y, planar.coords)
    for cols in ([0, 1], [0, 3, 2], [0, 1, 2, 3, 4]):
        got = e.global_criterion(cols)
        want = pb.indep_vars_criterion(cols)
        assert abs(got - want) <= 1e-9 * abs(want)


def test_full_aicc_search_matches_oracle():
    """Config-0 shape (adaptive bisquare, AICc golden search), smaller n."""
    pbm = datasets.config0(n=1200, seed=5)
    alg = GWRBasic()
    alg.setCoords(pbm.coords)
    alg.setDependentVariable(pbm.y)
    alg.setIndependentVariables(pbm.x)
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(0, True, BandwidthWeight.Bisquare), CRSDistance(False)))
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.AIC)
    betas = alg.fit()
    ref = O.gwr_fit(pbm.x, pbm.y, pbm.coords, adaptive=True, kernel=O.BISQUARE, autoselect_bandwidth=True,
                    criterion=O.AIC)
    assert alg.spatialWeight().weight().bandwidth() == ref["bandwidth"]
    got_list = alg.bandwidthSelectionCriterionList()
    assert [b for b, _ in got_list] == [b for b, _ in ref["bandwidth_criterion_list"]]
    for (_, a), (_, b) in zip(got_list, ref["bandwidth_criterion_list"]):
        assert abs(a - b) <= 1e-9 * abs(b)
    assert col_rel(betas, ref["betas"]) <= 1e-10
    d = alg.diagnostic()
    assert abs(d.AICc - ref["diagnostic"]["AICc"]) <= 1e-9 * abs(ref["diagnostic"]["AICc"])
    assert col_rel(alg.betasSE(), ref["betas_se"]) <= 1e-9


def test_fixed_cv_search_matches_oracle():
    """Config-1 shape (fixed gaussian, CV golden search over [0, maxDistance]), smaller n."""
    pbm = datasets.config1(n=1000, seed=6)
    alg = GWRBasic()
    alg.setCoords(pbm.coords)
    alg.setDependentVariable(pbm.y)
    alg.setIndependentVariables(pbm.x)
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(0, False, BandwidthWeight.Gaussian), CRSDistance(False)))
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.CV)
    betas = alg.fit()
    ref = O.gwr_fit(pbm.x, pbm.y, pbm.coords, adaptive=False, kernel=O.GAUSSIAN, autoselect_bandwidth=True,
                    criterion=O.CV)
    assert abs(alg.spatialWeight().weight().bandwidth() - ref["bandwidth"]) <= 1e-9 * ref["bandwidth"]
    assert col_rel(betas, ref["betas"]) <= 1e-9


def test_not_spd_is_dbl_max():
    """A collinear column makes every X^T W X singular: the criterion is DBL_MAX
    (GWRBasic.cpp:514-518) and the fit raises."""
    pbm = datasets.config0(n=300, seed=3)
    x = np.column_stack([pbm.x, pbm.x[:, 1] * 2.0])
    e = engine_for(x, pbm.y, pbm.coords)
    assert e.criterion(50, True, O.BISQUARE, O.AIC) == np.finfo(np.float64).max
    with pytest.raises(Exception):
        e.fit(50, True, O.BISQUARE, True)


def test_thresholds_reuse_cached_histograms(planar, geo, geo_rows):
    """Many bandwidths on one engine: later selects start from the cached
    per-row histograms and must stay bit-exact."""
    e = engine_for(planar.x, planar.y, planar.coords)
    pb = O.Problem(planar.x, planar.y, planar.coords)
    dists = [pb.distance_row(i) for i in range(pb.n)]
    for bw in (pb.n // 2, 25, pb.n // 5, 120.5, pb.n - 1, 64, pb.n + 10):
        got = e.thresholds(bw)
        want = np.array([O.adaptive_threshold(d, bw) for d in dists])
        assert np.array_equal(got, want), (bw, np.flatnonzero(got != want)[:5])
    g = engine_for(geo.x, geo.y, geo.coords, True)
    n = geo.n
    for bw in (n // 2, 25, n // 5, 120.5, n - 1, 64, n + 10):
        check_geo_thresholds(g.thresholds(bw), *geo_rows, bw)


def test_mixed_thresholds_close_to_exact(geo):
    """The mixed path selects on FP32 proxy distances: within 1e-5 relative."""
    e = engine_for(geo.x, geo.y, geo.coords, True)
    exact = e.thresholds(150)
    e.set_precision(1)
    approx = e.thresholds(150)
    assert np.max(np.abs(approx - exact) / exact) < 1e-5
