"""Batched evaluation of many GWR problems and bandwidth candidates
(include/gwgpu.h, gwgpu_batch_*).

    b = Batch(problems, precision=Precision.Mixed)
    b.set_candidates(cands)          # cands[q]: bandwidths of problem q
    b.autotune()                     # optional: pick the schedule on this batch
    values = b.evaluate()            # list of arrays, values[q][c]
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import BatchInfo, check, lib

_DP = ctypes.POINTER(ctypes.c_double)


def _ptrs(arrays):
    return (_DP * len(arrays))(*[a.ctypes.data_as(_DP) for a in arrays])


class Batch:
    def __init__(self, problems, precision=1, device=0):
        h = ctypes.c_void_p()
        check(lib().gwgpu_batch_create(int(device), ctypes.byref(h)))
        self._h = h
        self.problems = list(problems)
        xs = [np.asfortranarray(pb.x, dtype=np.float64) for pb in self.problems]
        ys = [np.ascontiguousarray(pb.y, dtype=np.float64) for pb in self.problems]
        cs = [np.asfortranarray(pb.coords, dtype=np.float64) for pb in self.problems]
        k = len(self.problems)
        n = (ctypes.c_int * k)(*[pb.n for pb in self.problems])
        p = (ctypes.c_int * k)(*[pb.p for pb in self.problems])
        g = (ctypes.c_int * k)(*[int(pb.geographic) for pb in self.problems])
        check(lib().gwgpu_batch_set_problems(self._h, k, n, p, _ptrs(xs), _ptrs(ys), _ptrs(cs), g, int(precision)))
        self.counts = None

    def close(self):
        if self._h:
            check(lib().gwgpu_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_candidates(self, cands, adaptive=True, kernel=2, criterion=0):
        cs = [np.ascontiguousarray(c, dtype=np.float64) for c in cands]
        self.counts = [len(c) for c in cs]
        cnt = (ctypes.c_int * len(cs))(*self.counts)
        check(lib().gwgpu_batch_set_candidates(self._h, cnt, _ptrs(cs), int(bool(adaptive)), int(kernel),
                                               int(criterion)))

    def evaluate(self, use_graph=True):
        total = sum(self.counts)
        out = np.zeros(total)
        check(lib().gwgpu_batch_evaluate(self._h, int(bool(use_graph)), out.ctypes.data_as(_DP)))
        res, o = [], 0
        for c in self.counts:
            res.append(out[o:o + c])
            o += c
        return res

    def autotune(self, repeats=3):
        check(lib().gwgpu_batch_autotune(self._h, int(repeats)))

    def set_tuning(self, flush_tiles=64, order=1, solve_rows=32, select_ctas=12):
        check(lib().gwgpu_batch_set_tuning(self._h, flush_tiles, order, solve_rows, select_ctas))

    def info(self):
        s = BatchInfo()
        check(lib().gwgpu_batch_get_info(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in BatchInfo._fields_}


__all__ = ["Batch"]
