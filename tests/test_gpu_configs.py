"""The FP64 drop-in against the oracle at the benchmark workloads' own sizes.

* config 0 exactly (n = 2,000, seed 0): the whole AICc golden search and fit;
* config-2 data (lon U(-10, 30), lat U(35, 60), p = 17, column scales 1e-2 ..
  1e3) at n = 3,000: the AICc search with great-circle distances against the
  libm oracle, plus grids with exact ties and data across the antimeridian;
* config 1 at n = 50,000: the CV golden search on the GPU, its criterion at the
  selected bandwidth against the oracle over every row, beta on a row subset;
* config 2 in FP64 at n = 200,000: thresholds and beta of a few hundred rows
  spread over the whole point set.

Bars as the reference's tests and the drop-in state them (GWRBasic.cpp outputs,
test/testGWRBasic.cpp:40-137): selected adaptive bandwidth identical, beta within
1e-10 relative (per column), AICc / CV within 1e-9 relative; great-circle
thresholds as parity_util states."""
import numpy as np
import pytest

import oracle as O
from libgwmodel_gb300 import BandwidthWeight, CRSDistance, Engine, GWRBasic, SpatialWeight, datasets
from parity_util import check_geo_thresholds, col_rel, geo_rows

pytestmark = pytest.mark.gpu


def facade_search(pb, criterion, adaptive=True, kernel=BandwidthWeight.Bisquare):
    alg = GWRBasic()
    alg.setCoords(pb.coords)
    alg.setDependentVariable(pb.y)
    alg.setIndependentVariables(pb.x)
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(0, adaptive, kernel), CRSDistance(pb.geographic)))
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(criterion)
    betas = alg.fit()
    return alg, betas


def check_search(alg, betas, ref):
    assert alg.spatialWeight().weight().bandwidth() == ref["bandwidth"]
    got_list = alg.bandwidthSelectionCriterionList()
    assert [b for b, _ in got_list] == [b for b, _ in ref["bandwidth_criterion_list"]]
    for (_, a), (_, b) in zip(got_list, ref["bandwidth_criterion_list"]):
        assert abs(a - b) <= 1e-9 * abs(b)
    assert col_rel(betas, ref["betas"]) <= 1e-10
    d = alg.diagnostic()
    assert abs(d.AICc - ref["diagnostic"]["AICc"]) <= 1e-9 * abs(ref["diagnostic"]["AICc"])
    assert col_rel(alg.betasSE(), ref["betas_se"]) <= 1e-9


def test_config0_full_search():
    """Config 0 as specified: n = 2,000, seed 0, adaptive bisquare, AICc search."""
    pb = datasets.config0()
    assert pb.n == 2000
    alg, betas = facade_search(pb, GWRBasic.AIC)
    ref = O.gwr_fit(pb.x, pb.y, pb.coords, adaptive=True, kernel=O.BISQUARE, autoselect_bandwidth=True,
                    criterion=O.AIC)
    check_search(alg, betas, ref)


def test_config2_shape_geographic_aicc_search():
    """Config-2 data (p = 17, column scales 1e-2 .. 1e3, great-circle) at n = 3,000:
    the AICc search picks the libm oracle's bandwidth through the same sequence."""
    pb = datasets.config2(n=3000, seed=22)
    alg, betas = facade_search(pb, GWRBasic.AIC)
    ref = O.gwr_fit(pb.x, pb.y, pb.coords, geographic=True, adaptive=True, kernel=O.BISQUARE,
                    autoselect_bandwidth=True, criterion=O.AIC)
    check_search(alg, betas, ref)


def _geo_problem(coords, seed, p=5):
    rng = np.random.default_rng(seed)
    n = len(coords)
    x = np.column_stack([np.ones(n), rng.standard_normal((n, p - 1))])
    beta = 1.0 + 0.5 * np.sin(np.radians(coords[:, :1]) * 3.0) * rng.uniform(-1, 1, (1, p))
    y = (x * beta).sum(1) + rng.normal(0, 0.3, n)
    return datasets.Problem("geo", np.asfortranarray(x), y, np.asfortranarray(coords), True, True, 2, 0, beta)


def _tie_grid():
    """Points on a 0.5-degree grid, several per node: many exactly equal distances."""
    rng = np.random.default_rng(31)
    lon = rng.integers(0, 40, 1600) * 0.5 - 5.0
    lat = rng.integers(0, 30, 1600) * 0.5 + 40.0
    return np.column_stack([lon, lat]).astype(np.float64)


def _antimeridian():
    """Points straddling lon = +-180 up to 89.9 degrees of latitude."""
    rng = np.random.default_rng(32)
    lon = rng.uniform(170, 190, 1600)
    lon = np.where(lon > 180, lon - 360, lon)
    lat = np.concatenate([rng.uniform(-30, 30, 1200), rng.uniform(80, 89.9, 400)])
    return np.column_stack([lon, lat])


@pytest.mark.parametrize("name,coords", [("ties", _tie_grid()), ("antimeridian", _antimeridian())])
def test_geographic_ties_and_antimeridian(name, coords, gc_host):
    pb = _geo_problem(coords, 33)
    libm, cr = geo_rows(pb.coords, range(pb.n), gc_host)
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, True)
    for bw in (20, 57, 200.5, 800, 1599, 1700):
        check_geo_thresholds(e.thresholds(bw), libm, cr, bw)
    alg, betas = facade_search(pb, GWRBasic.CV)
    ref = O.gwr_fit(pb.x, pb.y, pb.coords, geographic=True, adaptive=True, kernel=O.BISQUARE,
                    autoselect_bandwidth=True, criterion=O.CV)
    assert alg.spatialWeight().weight().bandwidth() == ref["bandwidth"], name
    assert col_rel(betas, ref["betas"]) <= 1e-10


def test_config1_full_size():
    """Config 1 at n = 50,000: fixed gaussian, CV golden search over [0, maxDistance].
    The CV score at the selected bandwidth is checked over all 50,000 rows, beta on 64."""
    pb = datasets.config1()
    assert pb.n == 50000
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, False)
    upper = e.max_distance()
    prob = O.Problem(pb.x, pb.y, pb.coords)
    assert upper == prob.max_distance()
    bw, crit_list = e.golden(False, O.GAUSSIAN, O.CV, 0.0, upper)
    got = e.criterion(bw, False, O.GAUSSIAN, O.CV)
    want, _ = prob.criterion(bw, False, O.GAUSSIAN, O.CV)
    assert abs(got - want) <= 1e-9 * abs(want), (bw, got, want)
    assert any(b == bw and abs(v - got) <= 1e-12 * abs(got) for b, v in crit_list)
    betas = e.fit(bw, False, O.GAUSSIAN, store_s=False)[0]
    rows = np.random.default_rng(41).choice(pb.n, 64, replace=False)
    ref = prob.predict(pb.coords[rows], bw, False, O.GAUSSIAN)
    assert col_rel(betas[rows], ref) <= 1e-10


def test_config2_fp64_full_size(gc_host):
    """Config 2 in FP64 at n = 200,000, p = 17: the thresholds of 256 rows spread
    over the point set (and so over all Hilbert blocks) at the selected bandwidth
    of the mixed bench (1351) and at the first golden point, and beta of those rows."""
    pb = datasets.config2()
    assert pb.n == 200000 and pb.p == 17
    rows = np.sort(np.random.default_rng(42).choice(pb.n, 256, replace=False))
    libm, cr = geo_rows(pb.coords, rows, gc_host)
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, True)
    for bw in (1351, float(np.floor(20 + (np.sqrt(5) - 1) / 2 * (pb.n - 20)))):
        check_geo_thresholds(e.thresholds(bw)[rows], libm, cr, bw)
    betas = e.fit(1351, True, O.BISQUARE, store_s=False)[0]
    prob = O.Problem(pb.x, pb.y, pb.coords, geographic=True)
    ref = prob.predict(pb.coords[rows], 1351, True, O.BISQUARE)
    assert col_rel(betas[rows], ref) <= 1e-10
