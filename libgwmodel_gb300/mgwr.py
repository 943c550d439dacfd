"""Python face of the GB300 multiscale GWR, mirroring ``gwm::GWRMultiscale``
(include/gwmodelpp/GWRMultiscale.h) so code written against the reference
reads the same::

    spatials = [SpatialWeight(BandwidthWeight(36, True, BandwidthWeight.Bisquare), CRSDistance(False))
                for _ in range(x.shape[1])]
    algorithm = GWRMultiscale()
    algorithm.setCoords(coords)
    algorithm.setDependentVariable(y)
    algorithm.setIndependentVariables(x)
    algorithm.setSpatialWeights(spatials)
    algorithm.setPreditorCentered([False, True, True])
    algorithm.setBandwidthInitilize([GWRMultiscale.Initial] * 3)
    algorithm.setBandwidthSelectionApproach([GWRMultiscale.AIC] * 3)
    algorithm.setBandwidthSelectThreshold([1e-5] * 3)
    algorithm.fit()
    [w.weight().bandwidth() for w in algorithm.spatialWeights()]

Every call goes through the C ABI of libgwgpu.so (gwgpu_mgwr_*) to the GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, dptr, iptr, lib
from .gwrbasic import (BandwidthWeight, CRSDistance, Logger, RegressionDiagnostic, SpatialWeight, _f64,
                       telegram_struct)


class GWRMultiscale:
    """gwm::GWRMultiscale on the GPU (GWRMultiscale.h:35)."""

    # BandwidthInitilizeType
    Null, Initial, Specified = 0, 1, 2
    # BandwidthSelectionCriterionType
    CV, AIC = 0, 1
    # BackFittingCriterionType
    CVR, dCVR = 0, 1

    def __init__(self, x=None, y=None, coords=None, spatialWeights=None):
        h = ctypes.c_void_p()
        check(lib().gwgpu_mgwr_create(ctypes.byref(h)))
        self._h = h
        self._p = 0
        self._n = 0
        self._sws = []
        self._telegram = None
        if x is not None:
            self.setIndependentVariables(x)
        if y is not None:
            self.setDependentVariable(y)
        if coords is not None:
            self.setCoords(coords)
        if spatialWeights is not None:
            self.setSpatialWeights(spatialWeights)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().gwgpu_mgwr_destroy(h)
            self._h = None

    # ------------------------------------------------------------ setters
    def setCoords(self, coords):
        c = _f64(coords)
        assert c.ndim == 2 and c.shape[1] == 2, "coords must be n x 2"
        check(lib().gwgpu_mgwr_set_coords(self._h, c.shape[0], dptr(c)))

    def setDependentVariable(self, y):
        v = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        check(lib().gwgpu_mgwr_set_dependent_variable(self._h, v.shape[0], dptr(v)))

    def setIndependentVariables(self, x):
        m = _f64(x)
        assert m.ndim == 2
        self._n, self._p = m.shape
        check(lib().gwgpu_mgwr_set_independent_variables(self._h, m.shape[0], m.shape[1], dptr(m)))

    def setSpatialWeights(self, sws):
        sws = [SpatialWeight(s.weight(), s.distance()) for s in sws]
        k = len(sws)
        bw = np.array([s.weight().bandwidth() for s in sws], dtype=np.float64)
        ad = np.array([int(s.weight().adaptive()) for s in sws], dtype=np.int32)
        ke = np.array([s.weight().kernel() for s in sws], dtype=np.int32)
        geo = {s.distance().geographic() for s in sws}
        if len(geo) > 1:
            raise ValueError("every spatial weight must use the same CRSDistance")
        check(lib().gwgpu_mgwr_set_spatial_weights(self._h, k, dptr(bw), iptr(ad), iptr(ke),
                                                   int(bool(geo.pop())) if geo else 0))
        self._sws = sws

    def _ints(self, fn, values):
        v = np.ascontiguousarray(np.asarray([int(t) for t in values], dtype=np.int32))
        check(fn(self._h, len(v), iptr(v)))

    def setBandwidthInitilize(self, types):
        self._ints(lib().gwgpu_mgwr_set_bandwidth_initilize, types)

    def setBandwidthSelectionApproach(self, approaches):
        self._ints(lib().gwgpu_mgwr_set_bandwidth_selection_approach, approaches)

    def setPreditorCentered(self, centered):
        self._ints(lib().gwgpu_mgwr_set_preditor_centered, [bool(c) for c in centered])

    def setBandwidthSelectThreshold(self, thresholds):
        v = np.ascontiguousarray(np.asarray(thresholds, dtype=np.float64))
        check(lib().gwgpu_mgwr_set_bandwidth_select_threshold(self._h, len(v), dptr(v)))

    def setBandwidthSelectRetryTimes(self, t):
        check(lib().gwgpu_mgwr_set_bandwidth_select_retry_times(self._h, int(t)))

    def setMaxIteration(self, m):
        check(lib().gwgpu_mgwr_set_max_iteration(self._h, int(m)))

    def setCriterionType(self, t):
        check(lib().gwgpu_mgwr_set_criterion_type(self._h, int(t)))

    def setCriterionThreshold(self, t):
        check(lib().gwgpu_mgwr_set_criterion_threshold(self._h, float(t)))

    def setAdaptiveLower(self, lower):
        check(lib().gwgpu_mgwr_set_adaptive_lower(self._h, int(lower)))

    def setGoldenUpperBounds(self, v):
        check(lib().gwgpu_mgwr_set_golden_upper_bounds(self._h, float(v)))

    def setGoldenLowerBounds(self, v):
        check(lib().gwgpu_mgwr_set_golden_lower_bounds(self._h, float(v)))

    def setHasHatMatrix(self, on):
        check(lib().gwgpu_mgwr_set_has_hat_matrix(self._h, int(bool(on))))

    def setHasIntercept(self, on):
        check(lib().gwgpu_mgwr_set_has_intercept(self._h, int(bool(on))))

    def setParallelType(self, t):
        check(lib().gwgpu_mgwr_set_parallel_type(self._h, int(t)))

    def setGPUId(self, g):
        check(lib().gwgpu_mgwr_set_gpu_id(self._h, int(g)))

    def setPrecision(self, p):
        check(lib().gwgpu_mgwr_set_precision(self._h, int(p)))

    def setTelegram(self, telegram: Logger):
        """setTelegram (Algorithm.h:164): messages, progress and cancellation."""
        if telegram is None:
            check(lib().gwgpu_mgwr_set_telegram(self._h, None))
            self._telegram = None
            return
        t = telegram_struct(telegram)
        self._telegram = (telegram, t)
        check(lib().gwgpu_mgwr_set_telegram(self._h, ctypes.byref(t)))

    # ------------------------------------------------------------ fit
    def fit(self):
        check(lib().gwgpu_mgwr_fit(self._h))
        return self.betas()

    def predict(self, locations):
        """GWRMultiscale::predict returns zeros (GWRMultiscale.h:601)."""
        return np.zeros((np.asarray(locations).shape[0], self._p), order="F")

    def status(self):
        return lib().gwgpu_mgwr_status(self._h)

    def _mat(self, fn):
        out = np.zeros((self._n, self._p), order="F")
        if out.size:
            check(fn(self._h, dptr(out)))
        return out

    def betas(self):
        return self._mat(lib().gwgpu_mgwr_betas)

    def betasSE(self):
        return self._mat(lib().gwgpu_mgwr_betas_se)

    def betasTV(self):
        return self._mat(lib().gwgpu_mgwr_betas_tv)

    def bandwidths(self):
        out = np.zeros(max(self._p, 1))
        check(lib().gwgpu_mgwr_bandwidths(self._h, dptr(out)))
        return out[:self._p]

    def spatialWeights(self):
        bws = self.bandwidths()
        return [SpatialWeight(BandwidthWeight(float(b), s.weight().adaptive(), s.weight().kernel()), s.distance())
                for b, s in zip(bws, self._sws)]

    def diagnostic(self) -> RegressionDiagnostic:
        out = np.zeros(7)
        check(lib().gwgpu_mgwr_diagnostic(self._h, dptr(out)))
        return RegressionDiagnostic(*out.tolist())

    def initialBandwidth(self):
        b, it = ctypes.c_double(), ctypes.c_int()
        check(lib().gwgpu_mgwr_info(self._h, ctypes.byref(b), ctypes.byref(it)))
        return b.value

    def iterations(self):
        b, it = ctypes.c_double(), ctypes.c_int()
        check(lib().gwgpu_mgwr_info(self._h, ctypes.byref(b), ctypes.byref(it)))
        return it.value

    def counters(self):
        """Work of the last fit: criterion evaluations, fits, hat updates, kernel
        launches and host seconds by phase (search, fit, hat)."""
        ll = [ctypes.c_longlong() for _ in range(4)]
        sec = np.zeros(3)
        check(lib().gwgpu_mgwr_counters(self._h, *[ctypes.byref(v) for v in ll], dptr(sec)))
        return {"criterion_evals": ll[0].value, "fits": ll[1].value, "hat_updates": ll[2].value,
                "kernel_launches": ll[3].value, "search_s": float(sec[0]), "fit_s": float(sec[1]),
                "hat_s": float(sec[2])}


__all__ = ["GWRMultiscale", "CRSDistance", "BandwidthWeight", "SpatialWeight"]
