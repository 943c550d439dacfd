"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the GWRBasic hot path.

The C restatement in ``gwr_oracle.c`` does the per-location work (distance,
kernel weight, local solve, criteria, final fit, golden-section search).  This
module builds it with gcc, binds it with ctypes and restates the orchestration
of ``GWRBasic::fit`` (GWRBasic.cpp:36-128) and ``VariableForwardSelector``
(VariableForwardSelector.cpp:9-91) on top.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this module, and only as the checker.  The product library never does.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgwr_oracle.so")
SOURCES = [os.path.join(HERE, "gwr_oracle.c")]
DEPS = SOURCES + [os.path.join(HERE, "gwr_oracle.h")]

DBL_MAX = np.finfo(np.float64).max
AIC, CV = 0, 1
GAUSSIAN, EXPONENTIAL, BISQUARE, TRICUBE, BOXCAR = range(5)

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc, OpenMP, no FP contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stale = force or not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(d) > os.path.getmtime(LIB_PATH) for d in DEPS)
    if stale:
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-D_GNU_SOURCE", "-o", tmp] + SOURCES + ["-lm"]
        subprocess.check_call(cmd)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Problem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("p", ctypes.c_int),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("coords", ctypes.c_void_p),
                ("geographic", ctypes.c_int), ("threads", ctypes.c_int)]


class _MgwrOpts(ctypes.Structure):
    _IP, _DP = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    _fields_ = [("adaptive", _IP), ("kernel", _IP), ("bw0", _DP), ("init_type", _IP), ("approach", _IP),
                ("centered", _IP), ("select_threshold", _DP), ("retry_times", ctypes.c_int),
                ("max_iteration", ctypes.c_int), ("criterion_type", ctypes.c_int),
                ("criterion_threshold", ctypes.c_double), ("adaptive_lower", ctypes.c_int),
                ("has_lower", ctypes.c_int), ("has_upper", ctypes.c_int), ("lower", ctypes.c_double),
                ("upper", ctypes.c_double), ("has_hat_matrix", ctypes.c_int), ("has_intercept", ctypes.c_int)]


class _MgwrOut(ctypes.Structure):
    _DP = ctypes.POINTER(ctypes.c_double)
    _fields_ = [("betas", _DP), ("betas_se", _DP), ("bws", _DP), ("init_bw", ctypes.c_double),
                ("shat", ctypes.c_double * 2), ("rss", ctypes.c_double), ("diag", ctypes.c_double * 6),
                ("iterations", ctypes.c_int)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            P = ctypes.POINTER(_Problem)
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int)
            d, i = ctypes.c_double, ctypes.c_int
            L.orc_gcdist_libm.restype = d
            L.orc_gcdist_libm.argtypes = [d, d, d, d]
            L.orc_distance_row.argtypes = [P, i, dp]
            L.orc_max_distance.restype = d
            L.orc_max_distance.argtypes = [P]
            L.orc_weight.restype = i
            L.orc_weight.argtypes = [dp, i, d, i, i, dp]
            L.orc_adaptive_threshold.restype = i
            L.orc_adaptive_threshold.argtypes = [dp, i, d, dp]
            L.orc_criterion.restype = d
            L.orc_criterion.argtypes = [P, d, i, i, i, dp]
            L.orc_criterion_rows.restype = d
            L.orc_criterion_rows.argtypes = [P, d, i, i, i, i, i]
            L.orc_indep_vars_criterion.restype = d
            L.orc_indep_vars_criterion.argtypes = [P, ip, i]
            L.orc_fit_core.restype = i
            L.orc_fit_core.argtypes = [P, d, i, i, i, dp, dp, dp, dp, dp]
            L.orc_predict.restype = i
            L.orc_predict.argtypes = [P, i, dp, d, i, i, dp]
            L.orc_mgwr_fit.restype = i
            L.orc_mgwr_fit.argtypes = [P, ctypes.POINTER(_MgwrOpts), ctypes.POINTER(_MgwrOut)]
            L.orc_golden.restype = i
            L.orc_golden.argtypes = [P, d, i, i, i, d, d, dp, dp, dp, i]
            L.orc_diagnostic.argtypes = [P, dp, dp, dp]
            L.orc_inv_sympd.restype = i
            L.orc_inv_sympd.argtypes = [dp, i]
            _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Problem:
    """Column-major copies of X, y and coords, like GWRBase/SpatialAlgorithm keep."""

    def __init__(self, x, y, coords, geographic=False, threads=None):
        self.x = np.asfortranarray(np.asarray(x, dtype=np.float64))
        self.y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        self.coords = np.asfortranarray(np.asarray(coords, dtype=np.float64))
        n, p = self.x.shape
        assert self.y.shape[0] == n and self.coords.shape == (n, 2)
        self.n, self.p = n, p
        self.geographic = bool(geographic)
        self.threads = int(threads or os.cpu_count() or 1)
        self._s = _Problem(n, p, self.x.ctypes.data, self.y.ctypes.data, self.coords.ctypes.data,
                           int(geographic), self.threads)

    def with_columns(self, cols):
        return Problem(self.x[:, cols], self.y, self.coords, self.geographic, self.threads)

    @property
    def ref(self):
        return ctypes.byref(self._s)

    def distance_row(self, i):
        out = np.empty(self.n)
        lib().orc_distance_row(self.ref, int(i), _dp(out))
        return out

    def max_distance(self):
        return lib().orc_max_distance(self.ref)

    def criterion(self, bw, adaptive, kernel, criterion):
        shat = np.zeros(2)
        v = lib().orc_criterion(self.ref, float(bw), int(adaptive), int(kernel), int(criterion), _dp(shat))
        return v, shat

    def criterion_rows(self, bw, adaptive, kernel, criterion, row0, row1):
        return lib().orc_criterion_rows(self.ref, float(bw), int(adaptive), int(kernel),
                                        int(criterion), int(row0), int(row1))

    def indep_vars_criterion(self, cols):
        c = np.ascontiguousarray(np.asarray(cols, dtype=np.int32))
        return lib().orc_indep_vars_criterion(self.ref, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                              len(c))

    def fit_core(self, bw, adaptive, kernel, store_s=True):
        n, p = self.n, self.p
        betas = np.zeros((n, p), order="F")
        se = np.zeros((n, p), order="F")
        shat = np.zeros(2)
        qdiag = np.zeros(n)
        S = np.zeros((n if store_s else 1, n), order="F")
        rc = lib().orc_fit_core(self.ref, float(bw), int(adaptive), int(kernel), int(store_s),
                                _dp(betas), _dp(se), _dp(shat), _dp(qdiag), _dp(S))
        if rc != 0:
            raise RuntimeError("inv_sympd(): matrix is singular or not positive definite")
        return betas, se, shat, qdiag, S

    def predict(self, locations, bw, adaptive, kernel):
        """GWRBasic::predictSerial: betas (nr x p) at the given locations."""
        loc = np.asfortranarray(locations, dtype=np.float64)
        nr = loc.shape[0]
        betas = np.zeros((nr, self.p), order="F")
        rc = lib().orc_predict(self.ref, nr, _dp(loc), float(bw), int(adaptive), int(kernel), _dp(betas))
        if rc != 0:
            raise RuntimeError("inv_sympd(): matrix is singular or not positive definite")
        return betas

    def mgwr(self, bw0, adaptive, kernel, init_type, approach, centered, select_threshold, retry_times=5,
             max_iteration=500, criterion_type=1, criterion_threshold=1e-6, adaptive_lower=10, lower=None,
             upper=None, hat_matrix=True, intercept=True):
        """GWRMultiscale::fit: per-variable lists (one entry per column of X).
        init_type 0 Null / 1 Initial / 2 Specified; approach 0 CV / 1 AIC;
        criterion_type 0 CVR / 1 dCVR.  Returns a dict of the outputs."""
        n, p = self.n, self.p
        ia = lambda v: (ctypes.c_int * p)(*[int(t) for t in v])
        da = lambda v: (ctypes.c_double * p)(*[float(t) for t in v])
        o = _MgwrOpts(ia(adaptive), ia(kernel), da(bw0), ia(init_type), ia(approach), ia(centered),
                      da(select_threshold), int(retry_times), int(max_iteration), int(criterion_type),
                      float(criterion_threshold), int(adaptive_lower), int(lower is not None),
                      int(upper is not None), float(lower or 0.0), float(upper or 0.0), int(hat_matrix),
                      int(intercept))
        betas = np.zeros((n, p), order="F")
        se = np.zeros((n, p), order="F")
        bws = np.zeros(p)
        out = _MgwrOut(_dp(betas), _dp(se), _dp(bws), 0.0, (ctypes.c_double * 2)(), 0.0, (ctypes.c_double * 6)(), 0)
        rc = lib().orc_mgwr_fit(self.ref, ctypes.byref(o), ctypes.byref(out))
        if rc != 0:
            raise RuntimeError(f"orc_mgwr_fit failed ({rc})")
        d = list(out.diag)
        return {"betas": betas, "betas_se": se, "bandwidths": bws, "init_bw": out.init_bw, "shat": list(out.shat),
                "rss": out.rss, "iterations": out.iterations,
                "diagnostic": dict(zip(["RSS", "AICc", "ENP", "EDF", "RSquare", "RSquareAdjust"], d))}

    def golden(self, bw0, adaptive, kernel, criterion, lower, upper, cap=512):
        bw = np.zeros(1)
        lb = np.zeros(cap)
        lf = np.zeros(cap)
        k = lib().orc_golden(self.ref, float(bw0), int(adaptive), int(kernel), int(criterion),
                             float(lower), float(upper), _dp(bw), _dp(lb), _dp(lf), cap)
        if k < 0:
            raise RuntimeError("Invalid initial values.")
        return float(bw[0]), list(zip(lb[:k].tolist(), lf[:k].tolist()))

    def diagnostic(self, betas, shat):
        out = np.zeros(7)
        b = np.asfortranarray(betas)
        s = np.ascontiguousarray(shat, dtype=np.float64)
        lib().orc_diagnostic(self.ref, _dp(b), _dp(s), _dp(out))
        return dict(zip(["RSS", "AIC", "AICc", "ENP", "EDF", "RSquare", "RSquareAdjust"], out.tolist()))


def adaptive_threshold(dist, bw):
    d = np.ascontiguousarray(dist, dtype=np.float64)
    out = np.zeros(1)
    rc = lib().orc_adaptive_threshold(_dp(d), len(d), float(bw), _dp(out))
    if rc != 0:
        raise IndexError("Mat::operator(): index out of bounds")
    return float(out[0])


def weight(dist, bw, adaptive, kernel):
    d = np.ascontiguousarray(dist, dtype=np.float64)
    w = np.zeros_like(d)
    if lib().orc_weight(_dp(d), len(d), float(bw), int(adaptive), int(kernel), _dp(w)) != 0:
        raise IndexError("Mat::operator(): index out of bounds")
    return w


def gcdist(lon1, lon2, lat1, lat2):
    """CRSDistance::SpGcdist (CRSDistance.cpp:15-69) with the platform libm."""
    return lib().orc_gcdist_libm(float(lon1), float(lon2), float(lat1), float(lat2))


def forward_select(pb: Problem, has_intercept: bool, threshold: float):
    """VariableForwardSelector::optimize (VariableForwardSelector.cpp:9-42) with
    GWRBasic::indepVarsSelectionCriterion (GWRBasic.cpp:309-346)."""
    variables = list(range(1 if has_intercept else 0, pb.p))

    def cols_of(index):
        v = [variables[i] for i in index]
        return ([0] if has_intercept else []) + v  # index2uvec (VariableForwardSelector.h)

    cur, rest = [], list(range(len(variables)))
    models = []
    for i in range(len(variables)):
        crit = []
        for j in range(len(rest)):
            cur.append(rest[j])
            aic = pb.indep_vars_criterion(cols_of(cur))
            crit.append(aic)
            models.append((list(cur), aic))
            cur.pop()
        best = int(np.argmin(crit))  # index_min: first minimum
        cur.append(rest[best])
        del rest[best]
    # sort(): each forward step's block sorted by criterion, descending (:52-64)
    tag = 0
    for size in range(len(variables), 0, -1):
        models[tag:tag + size] = sorted(models[tag:tag + size], key=lambda m: m[1], reverse=True)
        tag += size
    # select(): the last model whose predecessor is worse by >= threshold (:66-76)
    chosen = models[-1]
    for i in range(len(models) - 1, 0, -1):
        if models[i - 1][1] - models[i][1] >= threshold:
            chosen = models[i]
            break
    crit_list = [([variables[k] for k in m[0]], m[1]) for m in models]
    selected = [variables[k] for k in chosen[0]]
    return selected, crit_list


def gwr_fit(x, y, coords, *, geographic=False, bandwidth=0.0, adaptive=True, kernel=GAUSSIAN,
            autoselect_bandwidth=False, criterion=CV, golden_lower=None, golden_upper=None,
            has_hat_matrix=True, autoselect_vars=False, var_threshold=3.0, has_intercept=True,
            threads=None):
    """GWRBasic::fit (GWRBasic.cpp:36-128) with the OpenMP kernels.

    ``criterion`` follows the reference quirk that the criterion function
    pointer is CV until setBandwidthSelectionCriterion/setParallelType runs
    (GWRBasic.h:738-739); callers that never set it pass CV here.
    """
    pb = Problem(x, y, coords, geographic, threads)
    n = pb.n
    out = {}
    if autoselect_vars:
        selected, crit_list = forward_select(pb, has_intercept, var_threshold)
        out["selected_vars"] = selected
        out["var_criterion_list"] = crit_list
        if selected:
            cols = ([0] if has_intercept else []) + selected
            pb = pb.with_columns(cols)
    bw = float(bandwidth)
    if autoselect_bandwidth:
        lower = golden_lower if golden_lower is not None else (20.0 if adaptive else 0.0)
        upper = golden_upper if golden_upper is not None else (float(n) if adaptive else pb.max_distance())
        bw, crit = pb.golden(bw, adaptive, kernel, criterion, lower, upper)
        out["bandwidth_criterion_list"] = crit
    out["bandwidth"] = bw
    store_s = bool(has_hat_matrix) and n < 8192  # isStoreS (GWRBasic.h:708)
    betas, se, shat, qdiag, S = pb.fit_core(bw, adaptive, kernel, store_s)
    diag = pb.diagnostic(betas, shat)
    trS, trStS = shat
    sigma_hat = diag["RSS"] / (n - 2 * trS + trStS)
    out.update(betas=betas, betas_se=np.sqrt(sigma_hat * se), shat=shat, qdiag=qdiag, S=S,
               diagnostic=diag, x=pb.x)
    return out


def aicc(n, rss, trs):
    return n * math.log(rss / n) + n * math.log(2 * math.pi) + n * ((n + trs) / (n - 2 - trs))
