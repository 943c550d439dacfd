"""Python face of the GB300 GWRBasic engine, mirroring libgwmodel's API.

Names and argument meanings follow ``gwm::GWRBasic`` (include/gwmodelpp/
GWRBasic.h), ``CRSDistance``, ``BandwidthWeight`` and ``SpatialWeight`` so that
code written against the reference reads the same::

    distance = CRSDistance(False)
    bandwidth = BandwidthWeight(36, True, BandwidthWeight.Gaussian)
    algorithm = GWRBasic()
    algorithm.setCoords(coords)
    algorithm.setDependentVariable(y)
    algorithm.setIndependentVariables(x)
    algorithm.setSpatialWeight(SpatialWeight(bandwidth, distance))
    algorithm.fit()
    algorithm.diagnostic().AICc

Every call goes through the C ABI of libgwgpu.so to the GPU.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import GwgpuError, Stats, Telegram, check, dptr, iptr, lib


class ParallelType:
    SerialOnly = 1
    OpenMP = 2
    CUDA = 4


class Status:
    Success = 0
    Terminated = 1


class Precision:
    FP64 = 0
    Mixed = 1


class LogLevel:
    LOG_EMERG, LOG_ALERT, LOG_CRIT, LOG_ERR, LOG_WARNING, LOG_NOTICE, LOG_INFO, LOG_DEBUG = range(8)


class CRSDistance:
    """CRSDistance(isGeographic): planar Euclidean or WGS-84 great-circle (km)."""

    def __init__(self, isGeographic: bool = False):
        self._geographic = bool(isGeographic)

    def geographic(self):
        return self._geographic

    def setGeographic(self, g):
        self._geographic = bool(g)


class BandwidthWeight:
    """BandwidthWeight(size, adaptive, kernel) (BandwidthWeight.h:46-53)."""

    Gaussian, Exponential, Bisquare, Tricube, Boxcar = range(5)

    def __init__(self, size: float = 0.0, adaptive: bool = True, kernel: int = 0):
        self._bw, self._adaptive, self._kernel = float(size), bool(adaptive), int(kernel)

    def bandwidth(self):
        return self._bw

    def setBandwidth(self, v):
        self._bw = float(v)

    def adaptive(self):
        return self._adaptive

    def setAdaptive(self, v):
        self._adaptive = bool(v)

    def kernel(self):
        return self._kernel

    def setKernel(self, k):
        self._kernel = int(k)


class SpatialWeight:
    """SpatialWeight(weight, distance): deep copies of both (SpatialWeight.h:72-94)."""

    def __init__(self, weight: BandwidthWeight, distance: CRSDistance):
        self._w = BandwidthWeight(weight.bandwidth(), weight.adaptive(), weight.kernel())
        self._d = CRSDistance(distance.geographic())

    def weight(self):
        return self._w

    def distance(self):
        return self._d


@dataclass
class RegressionDiagnostic:
    RSS: float
    AIC: float
    AICc: float
    ENP: float
    EDF: float
    RSquare: float
    RSquareAdjust: float


class Logger:
    """ITelegram with no-op defaults (Logger.h:60-83); subclass to observe or cancel."""

    def print(self, message: str, level: int, fun_name: str, file_name: str):
        pass

    def progress(self, current: int, total: int, fun_name: str, file_name: str):
        pass

    def progress_percent(self, percent: float, fun_name: str, file_name: str):
        pass

    def stop(self) -> bool:
        return False


def telegram_struct(telegram: Logger) -> Telegram:
    """The C callbacks (gwgpu_telegram) of a Logger; keep the result alive while it is set."""

    def _print(_u, msg, level, fun, file):
        telegram.print(msg.decode(), level, fun.decode(), file.decode())

    def _progress(_u, cur, tot, fun, file):
        telegram.progress(int(cur), int(tot), fun.decode(), file.decode())

    def _percent(_u, pct, fun, file):
        telegram.progress_percent(float(pct), fun.decode(), file.decode())

    def _stop(_u):
        return 1 if telegram.stop() else 0

    return Telegram(None, Telegram.PRINT(_print), Telegram.PROGRESS(_progress), Telegram.PERCENT(_percent),
                    Telegram.STOP(_stop))


def _f64(a, shape=None):
    a = np.asarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return np.asfortranarray(a)


class GWRBasic:
    """gwm::GWRBasic on the GPU (GWRBasic.h:29)."""

    class BandwidthSelectionCriterionType:
        AIC = 0
        CV = 1

    AIC = 0
    CV = 1

    def __init__(self, x=None, y=None, coords=None, spatialWeight=None, hasHatMatrix=True, hasIntercept=True):
        h = ctypes.c_void_p()
        check(lib().gwgpu_gwr_create(ctypes.byref(h)))
        self._h = h
        self._keep = []
        self._telegram = None
        self._sw = None
        if x is not None:
            self.setIndependentVariables(x)
        if y is not None:
            self.setDependentVariable(y)
        if coords is not None:
            self.setCoords(coords)
        if spatialWeight is not None:
            self.setSpatialWeight(spatialWeight)
        self.setHasHatMatrix(hasHatMatrix)
        self.setHasIntercept(hasIntercept)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().gwgpu_gwr_destroy(h)
            self._h = None

    # ------------------------------------------------------------ setters
    def setCoords(self, coords):
        c = _f64(coords)
        assert c.ndim == 2 and c.shape[1] == 2, "coords must be n x 2"
        self._keep_coords = c
        check(lib().gwgpu_gwr_set_coords(self._h, c.shape[0], dptr(c)))

    def setDependentVariable(self, y):
        v = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        check(lib().gwgpu_gwr_set_dependent_variable(self._h, v.shape[0], dptr(v)))

    def setIndependentVariables(self, x):
        m = _f64(x)
        assert m.ndim == 2
        self._x = m
        check(lib().gwgpu_gwr_set_independent_variables(self._h, m.shape[0], m.shape[1], dptr(m)))

    def setSpatialWeight(self, sw: SpatialWeight):
        self._sw = sw
        w, d = sw.weight(), sw.distance()
        check(lib().gwgpu_gwr_set_spatial_weight(self._h, w.bandwidth(), int(w.adaptive()), w.kernel(),
                                                 int(d.geographic())))

    def setIsAutoselectBandwidth(self, on):
        check(lib().gwgpu_gwr_set_is_autoselect_bandwidth(self._h, int(bool(on))))

    def setBandwidthSelectionCriterion(self, criterion):
        check(lib().gwgpu_gwr_set_bandwidth_selection_criterion(self._h, int(criterion)))

    def setGoldenUpperBounds(self, v):
        check(lib().gwgpu_gwr_set_golden_upper_bounds(self._h, float(v)))

    def setGoldenLowerBounds(self, v):
        check(lib().gwgpu_gwr_set_golden_lower_bounds(self._h, float(v)))

    def setHasHatMatrix(self, on):
        check(lib().gwgpu_gwr_set_has_hat_matrix(self._h, int(bool(on))))

    def setHasIntercept(self, on):
        check(lib().gwgpu_gwr_set_has_intercept(self._h, int(bool(on))))

    def setIsAutoselectIndepVars(self, on):
        check(lib().gwgpu_gwr_set_is_autoselect_indep_vars(self._h, int(bool(on))))

    def setIndepVarSelectionThreshold(self, t):
        check(lib().gwgpu_gwr_set_indep_var_selection_threshold(self._h, float(t)))

    def setParallelType(self, t):
        check(lib().gwgpu_gwr_set_parallel_type(self._h, int(t)))

    def setOmpThreadNum(self, n):
        check(lib().gwgpu_gwr_set_omp_thread_num(self._h, int(n)))

    def setGPUId(self, g):
        check(lib().gwgpu_gwr_set_gpu_id(self._h, int(g)))

    def setGroupSize(self, s):
        check(lib().gwgpu_gwr_set_group_size(self._h, int(s)))

    def setPrecision(self, p):
        check(lib().gwgpu_gwr_set_precision(self._h, int(p)))

    def setTelegram(self, telegram: Logger):
        """setTelegram (Algorithm.h:164): messages, progress and cancellation."""
        if telegram is None:
            check(lib().gwgpu_gwr_set_telegram(self._h, None))
            self._telegram = None
            return

        t = telegram_struct(telegram)
        self._telegram = (telegram, t)
        check(lib().gwgpu_gwr_set_telegram(self._h, ctypes.byref(t)))

    # ------------------------------------------------------------ fit
    def fit(self):
        check(lib().gwgpu_gwr_fit(self._h))
        return self.betas()

    def predict(self, locations):
        """GWRBasic::predict: coefficients (nRp x p) at the given locations."""
        loc = np.asfortranarray(locations, dtype=np.float64)
        nr = loc.shape[0]
        check(lib().gwgpu_gwr_predict(self._h, nr, dptr(loc), None))
        return self.betas()

    def status(self):
        return lib().gwgpu_gwr_status(self._h)

    def _shape(self):
        n, p, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().gwgpu_gwr_shape(self._h, ctypes.byref(n), ctypes.byref(p), ctypes.byref(s)))
        return n.value, p.value, s.value

    def _mat(self, fn, rows, cols):
        out = np.zeros((rows, cols), order="F")
        if out.size:
            check(fn(self._h, dptr(out)))
        return out

    def betas(self):
        n, p, _ = self._shape()
        return self._mat(lib().gwgpu_gwr_betas, n, p)

    def betasSE(self):
        n, p, _ = self._shape()
        return self._mat(lib().gwgpu_gwr_betas_se, n, p)

    def sHat(self):
        out = np.zeros(2)
        n, _, _ = self._shape()
        if n:
            check(lib().gwgpu_gwr_shat(self._h, dptr(out)))
        return out

    def qDiag(self):
        n, _, _ = self._shape()
        return self._mat(lib().gwgpu_gwr_qdiag, n, 1).reshape(-1)

    def s(self):
        n, _, sr = self._shape()
        return self._mat(lib().gwgpu_gwr_s, sr, n)

    def diagnostic(self) -> RegressionDiagnostic:
        out = np.zeros(7)
        check(lib().gwgpu_gwr_diagnostic(self._h, dptr(out)))
        return RegressionDiagnostic(*out.tolist())

    def bandwidth(self):
        b = ctypes.c_double()
        check(lib().gwgpu_gwr_bandwidth(self._h, ctypes.byref(b)))
        return b.value

    def spatialWeight(self) -> SpatialWeight:
        sw = self._sw or SpatialWeight(BandwidthWeight(), CRSDistance())
        w = sw.weight()
        return SpatialWeight(BandwidthWeight(self.bandwidth(), w.adaptive(), w.kernel()), sw.distance())

    def bandwidthSelectionCriterionList(self):
        c = ctypes.c_int()
        check(lib().gwgpu_gwr_bandwidth_criterion_list(self._h, ctypes.byref(c), None, None))
        bw, val = np.zeros(max(c.value, 1)), np.zeros(max(c.value, 1))
        check(lib().gwgpu_gwr_bandwidth_criterion_list(self._h, ctypes.byref(c), dptr(bw), dptr(val)))
        return list(zip(bw[:c.value].tolist(), val[:c.value].tolist()))

    def selectedVariables(self):
        c = ctypes.c_int()
        check(lib().gwgpu_gwr_selected_vars(self._h, ctypes.byref(c), None))
        v = np.zeros(max(c.value, 1), dtype=np.int32)
        check(lib().gwgpu_gwr_selected_vars(self._h, ctypes.byref(c), iptr(v)))
        return v[:c.value].tolist()

    def indepVarsSelectionCriterionList(self):
        c, tot = ctypes.c_int(), ctypes.c_int()
        check(lib().gwgpu_gwr_var_criterion_list(self._h, ctypes.byref(c), ctypes.byref(tot), None, None, None))
        lens = np.zeros(max(c.value, 1), dtype=np.int32)
        vars_ = np.zeros(max(tot.value, 1), dtype=np.int32)
        vals = np.zeros(max(c.value, 1))
        check(lib().gwgpu_gwr_var_criterion_list(self._h, ctypes.byref(c), ctypes.byref(tot), iptr(lens),
                                                 iptr(vars_), dptr(vals)))
        out, off = [], 0
        for i in range(c.value):
            out.append((vars_[off:off + lens[i]].tolist(), float(vals[i])))
            off += lens[i]
        return out


class Engine:
    """The engine primitives (gwgpu_engine_*): one criterion, the final fit, thresholds."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().gwgpu_engine_create(int(device), ctypes.byref(h)))
        self._h = h
        self.n = self.p = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().gwgpu_engine_destroy(h)
            self._h = None

    def set_data(self, x, y, coords, geographic=False):
        self._x = _f64(x)
        self._y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        self._c = _f64(coords)
        self.n, self.p = self._x.shape
        check(lib().gwgpu_engine_set_data(self._h, self.n, self.p, dptr(self._x), dptr(self._y), dptr(self._c),
                                          int(bool(geographic))))

    def set_precision(self, p):
        check(lib().gwgpu_engine_set_precision(self._h, int(p)))

    def set_refinement(self, steps, refine_search=False):
        check(lib().gwgpu_engine_set_refinement(self._h, int(steps), int(bool(refine_search))))

    def set_flush_tiles(self, tiles):
        check(lib().gwgpu_engine_set_flush_tiles(self._h, int(tiles)))

    def set_tc_wait_limit(self, polls):
        """Polls of each pipeline wait of the tensor-core contraction (0: default);
        small values exercise the timeout path."""
        check(lib().gwgpu_engine_set_tc_wait_limit(self._h, int(polls)))

    def criterion(self, bw, adaptive, kernel, criterion):
        v = ctypes.c_double()
        check(lib().gwgpu_engine_criterion(self._h, float(bw), int(bool(adaptive)), int(kernel), int(criterion),
                                           ctypes.byref(v)))
        return v.value

    def global_criterion(self, cols):
        c = np.ascontiguousarray(np.asarray(cols, dtype=np.int32))
        v = ctypes.c_double()
        check(lib().gwgpu_engine_global_criterion(self._h, len(c), iptr(c), ctypes.byref(v)))
        return v.value

    def fit(self, bw, adaptive, kernel, store_s=True):
        n, p = self.n, self.p
        betas = np.zeros((n, p), order="F")
        se = np.zeros((n, p), order="F")
        shat = np.zeros(2)
        qdiag = np.zeros(n)
        S = np.zeros((n if store_s else 1, n), order="F")
        check(lib().gwgpu_engine_fit(self._h, float(bw), int(bool(adaptive)), int(kernel), int(bool(store_s)),
                                     dptr(betas), dptr(se), dptr(shat), dptr(qdiag), dptr(S)))
        return betas, se, shat, qdiag, S

    def predict(self, locations, bw, adaptive, kernel):
        loc = np.asfortranarray(locations, dtype=np.float64)
        nr = loc.shape[0]
        out = np.zeros((nr, self.p), order="F")
        check(lib().gwgpu_engine_predict(self._h, nr, dptr(loc), float(bw), int(bool(adaptive)), int(kernel),
                                         dptr(out)))
        return out

    def max_distance(self):
        v = ctypes.c_double()
        check(lib().gwgpu_engine_max_distance(self._h, ctypes.byref(v)))
        return v.value

    def golden(self, adaptive, kernel, criterion, lower, upper, cap=512):
        """Golden-section bandwidth search on the resident data: (bandwidth, [(bw, criterion), ...])."""
        bw = ctypes.c_double()
        cnt = ctypes.c_int()
        lb, lv = np.zeros(cap), np.zeros(cap)
        check(lib().gwgpu_engine_golden(self._h, int(bool(adaptive)), int(kernel), int(criterion), float(lower),
                                        float(upper), ctypes.byref(bw), ctypes.byref(cnt), dptr(lb), dptr(lv), cap))
        k = min(cnt.value, cap)
        return bw.value, list(zip(lb[:k].tolist(), lv[:k].tolist()))

    def clear_cache(self):
        check(lib().gwgpu_engine_clear_cache(self._h))

    def set_distance_cache(self, limit_bytes=-1):
        """Distance cache of the mixed geographic contraction: -1 automatic
        (default), 0 never, > 0 at most that many bytes (it takes n^2 x 4)."""
        check(lib().gwgpu_engine_set_distance_cache(self._h, int(limit_bytes)))

    def release_distance_cache(self):
        """Free the device's distance cache if this engine owns it."""
        check(lib().gwgpu_engine_release_distance_cache(self._h))

    def distance_cache_active(self):
        v = ctypes.c_int(0)
        check(lib().gwgpu_engine_distance_cache_active(self._h, ctypes.byref(v)))
        return bool(v.value)

    def record_event(self, slot):
        check(lib().gwgpu_engine_event_record(self._h, int(slot)))

    def elapsed_ms(self, first, second):
        ms = ctypes.c_float()
        check(lib().gwgpu_engine_event_elapsed(self._h, int(first), int(second), ctypes.byref(ms)))
        return ms.value

    def thresholds(self, bw, adaptive=True):
        out = np.zeros(self.n)
        check(lib().gwgpu_engine_thresholds(self._h, float(bw), int(bool(adaptive)), dptr(out)))
        return out

    def enable_stats(self, on=True, phases=False):
        """Event timings and counters; phases=True adds the contraction's
        clock64 phase counters (instrumented kernels, profiling only)."""
        check(lib().gwgpu_engine_enable_stats(self._h, (2 if phases else 1) if on else 0))

    def stats(self):
        s = Stats()
        check(lib().gwgpu_engine_get_stats(self._h, ctypes.byref(s)))
        out = {k: getattr(s, k) for k, _ in Stats._fields_}
        out["contract_phase_cycles"] = list(out["contract_phase_cycles"])
        return out

    def reset_stats(self):
        check(lib().gwgpu_engine_reset_stats(self._h))

    def tc_selftest(self, A, B):
        """D = A B^T on the tensor cores (A: 128 x 32, B: N x 32, float32)."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        B = np.ascontiguousarray(B, dtype=np.float32)
        N = B.shape[0]
        D = np.zeros((128, N), dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        check(lib().gwgpu_engine_tc_selftest(self._h, N, A.ctypes.data_as(fp), B.ctypes.data_as(fp),
                                             D.ctypes.data_as(fp)))
        return D


__all__ = ["GWRBasic", "CRSDistance", "BandwidthWeight", "SpatialWeight", "RegressionDiagnostic", "Logger",
           "ParallelType", "Status", "Precision", "LogLevel", "Engine", "GwgpuError"]
