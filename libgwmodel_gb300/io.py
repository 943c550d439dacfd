"""CSV input through the library's native reader (gwgpu_csv_read): a header
row of column names (quoted or not) and numeric rows, parsed on all host
threads into column-major arrays ready for the setters::

    t = read_csv("londonhp100data.csv")
    x = t.columns(["FLOORSZ", "PROF"])     # n x 2, Fortran order
    y = t.column("PURCHASE")
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, dptr, lib


class Table:
    """A parsed CSV (gwgpu_table)."""

    def __init__(self, handle):
        self._h = handle
        r, c = ctypes.c_int(), ctypes.c_int()
        check(lib().gwgpu_table_shape(self._h, ctypes.byref(r), ctypes.byref(c)))
        self.rows, self.cols = r.value, c.value
        self.names = [lib().gwgpu_table_column_name(self._h, k).decode() for k in range(self.cols)]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().gwgpu_table_destroy(h)
            self._h = None

    def columns(self, names=None):
        """The named columns (all by default) as a rows x k column-major array."""
        names = list(self.names if names is None else names)
        out = np.zeros((self.rows, len(names)), order="F")
        arr = (ctypes.c_char_p * max(len(names), 1))(*[n.encode() for n in names])
        if names:
            check(lib().gwgpu_table_columns(self._h, len(names), arr, dptr(out)))
        return out

    def column(self, name):
        return self.columns([name])[:, 0].copy()


def read_csv(path) -> Table:
    h = ctypes.c_void_p()
    check(lib().gwgpu_csv_read(str(path).encode(), ctypes.byref(h)))
    return Table(h)


__all__ = ["Table", "read_csv"]
