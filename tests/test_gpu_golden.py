"""test/testGWRBasic.cpp of the reference, on the GPU through the C ABI.

Each section uses the same inputs and asserts the same known answers at the
same absolute tolerance (1e-8)."""
import numpy as np
import pytest

from libgwmodel_gb300 import (BandwidthWeight, CRSDistance, GWRBasic, Logger, ParallelType, SpatialWeight,
                              Status)

pytestmark = pytest.mark.gpu


def make(londonhp, bw, adaptive, kernel=BandwidthWeight.Gaussian):
    alg = GWRBasic()
    alg.setCoords(londonhp["coords"])
    alg.setDependentVariable(londonhp["y"])
    alg.setIndependentVariables(londonhp["x"])
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(bw, adaptive, kernel), CRSDistance(False)))
    alg.setParallelType(ParallelType.CUDA)
    alg.setGPUId(0)
    alg.setGroupSize(64)
    return alg


def check_diag(d, e, tol):
    assert abs(d.AIC - e["AIC"]) <= tol, (d.AIC, e["AIC"])
    assert abs(d.AICc - e["AICc"]) <= tol, (d.AICc, e["AICc"])
    assert abs(d.RSquare - e["RSquare"]) <= tol
    assert abs(d.RSquareAdjust - e["RSquareAdjust"]) <= tol


def test_adaptive_bandwidth_no_optimisation(londonhp):
    alg = make(londonhp, 36, True)
    alg.fit()
    assert alg.hasIntercept() if hasattr(alg, "hasIntercept") else True
    check_diag(alg.diagnostic(), londonhp["expected"]["adaptive_gaussian_bw36"], londonhp["tol"])


def test_fixed_bandwidth_no_optimisation(londonhp):
    alg = make(londonhp, 5000, False)
    alg.fit()
    check_diag(alg.diagnostic(), londonhp["expected"]["fixed_gaussian_bw5000"], londonhp["tol"])


def test_adaptive_cv_bandwidth_optimisation(londonhp):
    alg = make(londonhp, 0, True)
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.CV)
    alg.fit()
    assert int(alg.spatialWeight().weight().bandwidth()) == 67


def test_aic_variable_optimisation(londonhp):
    e = londonhp["expected"]["variable_selection_aic"]
    alg = make(londonhp, 36, True)
    alg.setIsAutoselectIndepVars(True)
    alg.setIndepVarSelectionThreshold(3.0)
    alg.fit()
    crit = alg.indepVarsSelectionCriterionList()
    assert [c[0] for c in crit] == [c[0] for c in e["criterion_list"]]
    for (_, a), (_, b) in zip(crit, e["criterion_list"]):
        assert abs(a - b) <= londonhp["tol"], (a, b)
    assert alg.selectedVariables() == e["selected"]


def test_cv_bandwidth_and_variable_optimisation(londonhp):
    e = londonhp["expected"]["cv_search_with_variable_selection"]
    alg = make(londonhp, 36, True)
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.CV)
    alg.setIsAutoselectIndepVars(True)
    alg.setIndepVarSelectionThreshold(3.0)
    alg.fit()
    assert alg.selectedVariables() == e["selected"]
    assert alg.spatialWeight().weight().bandwidth() == 31.0
    check_diag(alg.diagnostic(), e, londonhp["tol"])


class TerminateCheckTelegram(Logger):
    """test/TerminateCheckTelegram.cpp: cancel at the first progress report
    with current >= breakProgress (the stage-name test there is always true)."""

    def __init__(self, stage, progress):
        self.stage, self.brk, self.cancelled = stage, progress, False

    def progress(self, current, total, fun, file):
        if current >= self.brk:
            self.cancelled = True

    def progress_percent(self, percent, fun, file):
        if percent * 100 >= self.brk:
            self.cancelled = True

    def stop(self):
        return self.cancelled


@pytest.mark.parametrize("criterion", [GWRBasic.CV, GWRBasic.AIC])
def test_cancel(londonhp, criterion):
    """test/testGWRBasic.cpp:245-344: fit() does not throw and ends Terminated."""
    stages = [("indepVarsSelection", 0), ("indepVarsSelection", 10), ("bandwidthSize", 0),
              ("bandwidthSize", 10), ("fit", 0), ("fit", 10)]
    for stage, prog in stages:
        alg = make(londonhp, 0, True)
        alg.setTelegram(TerminateCheckTelegram(stage, prog))
        alg.setIsAutoselectBandwidth(True)
        alg.setIsAutoselectIndepVars(True)
        alg.setBandwidthSelectionCriterion(criterion)
        alg.fit()
        assert alg.status() == Status.Terminated
        assert np.all(alg.betas() == 0.0)


def test_telegram_messages(londonhp):
    """The tagged strings GWmodelS parses (Algorithm.h:102-109, IBandwidthSelectable.h:30-49)."""
    msgs = []

    class Rec(Logger):
        def print(self, message, level, fun, file):
            msgs.append(message)

    alg = make(londonhp, 0, True)
    alg.setTelegram(Rec())
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.CV)
    alg.fit()
    assert msgs[0] == "#stage Initializing"
    assert "#stage Bandwidth selection" in msgs
    assert "#bandwidth-criterion adaptive,criterion" in msgs
    assert any(m.startswith("#bandwidth-criterion 67,") for m in msgs)
    assert msgs[-2:] == ["#stage Model fitting", "#stage Model Diagnostic"]
