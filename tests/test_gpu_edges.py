"""Edge inputs of the FP64 drop-in against the oracle: the widest X the engine
takes (p = 25: Z has 350 columns, more than one contraction launch covers),
geographic data across the antimeridian and at high latitude, and the smallest
problems.  Bars as in test_gpu_parity: thresholds bit-exact (great-circle
ones as parity_util states), beta within 1e-10 of each column's scale,
criteria within 1e-9 relative."""
import numpy as np
import pytest

import oracle as O
from libgwmodel_gb300 import Engine, Precision
from parity_util import check_geo_thresholds, geo_rows

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def col_rel(a, b):
    return max(rel(a[:, k], b[:, k]) for k in range(b.shape[1]))


def problem(n, p, coords, seed):
    rng = np.random.default_rng(seed)
    x = np.column_stack([np.ones(n), rng.standard_normal((n, p - 1))])
    beta = rng.uniform(-2, 2, p)
    y = x @ beta + rng.normal(0, 0.5, n)
    return np.asfortranarray(x), y, np.asfortranarray(coords)


def check_against_oracle(x, y, coords, geographic, bw, adaptive, kernel, criterion=O.AIC):
    e = Engine(0)
    e.set_data(x, y, coords, geographic)
    pb = O.Problem(x, y, coords, geographic=geographic)
    got = e.criterion(bw, adaptive, kernel, criterion)
    want = pb.criterion(bw, adaptive, kernel, criterion)[0]
    assert abs(got - want) <= 1e-9 * abs(want), (got, want)
    b, se, shat, q, S = e.fit(bw, adaptive, kernel, True)
    rb, rse, rshat, rq, rS = pb.fit_core(bw, adaptive, kernel, True)
    assert col_rel(b, rb) <= 1e-10
    assert col_rel(se, rse) <= 1e-9
    assert rel(shat, rshat) <= 1e-9
    assert rel(q, rq) <= 1e-9
    return e, pb


def test_widest_x_takes_several_contraction_launches():
    rng = np.random.default_rng(40)
    n, p = 900, 25
    x, y, c = problem(n, p, rng.uniform(0, 100, (n, 2)), 41)
    check_against_oracle(x, y, c, False, 300, True, O.BISQUARE)
    check_against_oracle(x, y, c, False, 35.0, False, O.GAUSSIAN)


@pytest.mark.parametrize("bw", [25, 180.5])
def test_antimeridian_and_high_latitude(bw, gc_host):
    """Longitudes on both sides of +-180 and latitudes up to 89.9 degrees."""
    rng = np.random.default_rng(42)
    n = 700
    lon = rng.uniform(170, 190, n)
    lon = np.where(lon > 180, lon - 360, lon)
    lat = rng.uniform(60, 89.9, n)
    x, y, c = problem(n, 4, np.column_stack([lon, lat]), 43)
    e, pb = check_against_oracle(x, y, c, True, bw, True, O.BISQUARE)
    check_geo_thresholds(e.thresholds(bw), *geo_rows(c, range(n), gc_host), bw)
    # the mixed path on the same data: within its tolerance of FP64
    e.set_precision(Precision.Mixed)
    got = e.criterion(bw, True, O.BISQUARE, O.AIC)
    ref = pb.criterion(bw, True, O.BISQUARE, O.AIC)[0]
    assert abs(got - ref) <= 1e-5 * abs(ref)


def test_whole_sphere_smallest_and_largest_ranks(gc_host):
    """25,003 points over the whole sphere, so dozens of pairs lie within
    4e-4 rad of each other's antipode: the FP32 proxy of such a pair keeps its
    precision (the exact select's band around it holds), and a window that
    reaches past 19,200 km still classifies tiles below it correctly.  Rows:
    the 24 whose nearest antipodal neighbour is closest, and 24 at random."""
    rng = np.random.default_rng(44)
    n = 25003
    lon = rng.uniform(-180.0, 180.0, n)
    lat = np.degrees(np.arcsin(rng.uniform(-0.999, 0.999, n)))
    x, y, c = problem(n, 3, np.column_stack([lon, lat]), 45)
    lo, la = np.radians(c[:, 0]), np.radians(c[:, 1])
    u = np.column_stack([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la)])
    anti = np.concatenate([np.max(-(u[s:s + 2048] @ u.T), axis=1) for s in range(0, n, 2048)])
    rows = sorted(set(np.argsort(-anti)[:24].tolist()) | set(rng.choice(n, 24, replace=False).tolist()))
    assert anti[rows].max() > 1.0 - 2e-8  # a pair within 2e-4 rad of the antipode
    libm, cr = geo_rows(c, rows, gc_host)
    e = Engine(0)
    e.set_data(x, y, c, True)
    m = Engine(0)
    m.set_data(x, y, c, True)
    m.set_precision(Precision.Mixed)
    for bw in (2, 25, 4000, n - 1):
        got = e.thresholds(bw)
        check_geo_thresholds(got[rows], libm, cr, bw)
        mixed = m.thresholds(bw)
        assert np.max(np.abs(mixed - got) / got) <= 1e-5, bw


@pytest.mark.parametrize("n", [3, 4, 5])
def test_smallest_problems(n):
    """At n = 3 a boxcar of 3 neighbours leaves 2 points for 2 coefficients: an
    exact fit whose RSS is rounding noise, so only the gaussian case is compared."""
    rng = np.random.default_rng(44 + n)
    x, y, c = problem(n, 2, rng.uniform(0, 10, (n, 2)), 50 + n)
    if n > 3:
        check_against_oracle(x, y, c, False, n, True, O.BOXCAR)  # every nearer neighbour at weight 1
    check_against_oracle(x, y, c, False, 50.0, False, O.GAUSSIAN)


@pytest.mark.parametrize("p", [1, 2, 19, 20, 21])
@pytest.mark.parametrize("criterion", [O.AIC, O.CV])
def test_criterion_solve_forms_at_their_column_limits(p, criterion):
    """The criterion without beta runs one location per thread up to p = 20 and
    one warp per location beyond; both agree with the oracle at the edges
    (p = 1 has no off-diagonal work, p = 20 fills the per-thread factor)."""
    rng = np.random.default_rng(100 + p)
    n = 700
    c = rng.uniform(0, 100, (n, 2))
    x, y, c = problem(n, p, c, 200 + p)
    e = Engine(0)
    e.set_data(x, y, c, False)
    pb = O.Problem(x, y, c, geographic=False)
    for bw, adaptive, kernel in ((max(3 * p, 60), True, O.BISQUARE), (40.0, False, O.GAUSSIAN)):
        got = e.criterion(bw, adaptive, kernel, criterion)
        want = pb.criterion(bw, adaptive, kernel, criterion)[0]
        assert abs(got - want) <= 1e-9 * abs(want), (p, bw, got, want)
