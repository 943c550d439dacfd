"""The serving loop (include/gwgpu.h, gwgpu_server_*) from Python.

    srv = Server(device=0, hbm_budget_gb=150, slots=8)
    rid = srv.submit(problem, kind=SEARCH, precision=Precision.Mixed)
    res, betas = srv.wait(rid)

Requests are copied at submit, admitted first come first served as slots and
the HBM budget allow, and run concurrently on the device; ``run_stream``
replays a timed request stream and reports latency percentiles.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from ._lib import GwgpuError, Request, Result, ServerStats, check, dptr, lib

FIT, SEARCH = 0, 1


class Server:
    def __init__(self, device=0, hbm_budget_gb=150.0, slots=8):
        h = ctypes.c_void_p()
        check(lib().gwgpu_server_create(int(device), float(hbm_budget_gb) * 1e9, int(slots), ctypes.byref(h)))
        self._h = h
        self._keep = {}
        self._lock = threading.Lock()

    def close(self):
        if self._h:
            check(lib().gwgpu_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, pb, kind=FIT, bandwidth=0.0, precision=1, adaptive=None, kernel=None, criterion=None):
        """Queue one request; returns its id.  The data are copied by the call."""
        x = np.asfortranarray(pb.x, dtype=np.float64)
        y = np.ascontiguousarray(pb.y, dtype=np.float64)
        c = np.asfortranarray(pb.coords, dtype=np.float64)
        betas = np.zeros((pb.n, pb.p), order="F")
        r = Request(pb.n, pb.p, dptr(c), dptr(x), dptr(y), int(pb.geographic), int(kind),
                    int(pb.adaptive if adaptive is None else adaptive), int(pb.kernel if kernel is None else kernel),
                    int(pb.criterion if criterion is None else criterion), float(bandwidth), int(precision))
        rid = ctypes.c_longlong()
        check(lib().gwgpu_server_submit(self._h, ctypes.byref(r), dptr(betas), ctypes.byref(rid)))
        with self._lock:
            self._keep[rid.value] = betas
        return rid.value

    def estimate(self, pb, kind=FIT, bandwidth=0.0, precision=1):
        """Bytes this server admits such a request with."""
        x = np.asfortranarray(pb.x, dtype=np.float64)
        y = np.ascontiguousarray(pb.y, dtype=np.float64)
        c = np.asfortranarray(pb.coords, dtype=np.float64)
        r = Request(pb.n, pb.p, dptr(c), dptr(x), dptr(y), int(pb.geographic), int(kind), int(pb.adaptive),
                    int(pb.kernel), int(pb.criterion), float(bandwidth), int(precision))
        return lib().gwgpu_server_estimate(self._h, ctypes.byref(r))

    def wait(self, rid, timeout_ms=-1.0):
        res = Result()
        check(lib().gwgpu_server_wait(self._h, ctypes.c_longlong(rid), float(timeout_ms), ctypes.byref(res)))
        with self._lock:
            betas = self._keep.pop(rid)
        return res, betas

    def stats(self):
        s = ServerStats()
        check(lib().gwgpu_server_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}


def result_dict(res):
    return {"status": res.status, "slot": res.slot, "evaluations": res.evaluations, "bandwidth": res.bandwidth,
            "aicc": res.aicc, "rss": res.rss, "shat": [res.shat[0], res.shat[1]], "submit_ms": res.submit_ms,
            "start_ms": res.start_ms, "end_ms": res.end_ms, "error": res.error.decode(errors="replace")}


def run_stream(server, requests, precision=1):
    """Submit each request at its arrival time (seconds from now) from a
    feeder thread, wait for all, and return per-request results."""
    ids = [None] * len(requests)
    t0 = time.perf_counter()

    def feed():
        for k, rq in enumerate(requests):
            delay = rq.arrival_s - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids[k] = server.submit(rq.problem, kind=rq.kind, bandwidth=rq.bandwidth, precision=precision)

    th = threading.Thread(target=feed)
    th.start()
    th.join()
    out = []
    for k, rq in enumerate(requests):
        res, betas = server.wait(ids[k])
        out.append((result_dict(res), betas))
    return out, time.perf_counter() - t0


def percentile(v, q):
    v = np.sort(np.asarray(v, dtype=np.float64))
    if v.size == 0:
        return 0.0
    return float(np.percentile(v, q))


__all__ = ["Server", "FIT", "SEARCH", "run_stream", "result_dict", "percentile", "GwgpuError"]
