"""Shared checks of the GPU engine against the oracle (imported by the tests).

Great-circle distances: the engine evaluates the reference's formula
(CRSDistance.cpp:15-69) with correctly rounded sin/cos/atan, the oracle with
the platform libm, which rounds a small fraction of results the other way.
Adaptive thresholds are therefore held bit-exact to the order statistics of
the engine's own distances recomputed on the host (the select is exact, ties
included), and against libm to the stated bar: at most GEO_THR_FRAC of the
thresholds different, each by at most GEO_THR_ULP ulp, and identical
neighbour sets {j : d_ij < thr_i} in every row except for points whose libm
distance lies within GEO_THR_ULP ulp of the threshold (a near-tie that the two
roundings order differently; on random data the sets are identical)."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np

import oracle as O

GEO_THR_FRAC = 0.03
GEO_THR_ULP = 8


def ulps(a, b):
    a = np.atleast_1d(np.asarray(a, np.float64)).view(np.int64)
    b = np.atleast_1d(np.asarray(b, np.float64)).view(np.int64)
    return np.abs(a - b)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def col_rel(a, b):
    return max(rel(a[:, k], b[:, k]) for k in range(b.shape[1]))


def geo_rows(coords, rows, gc_host):
    """Distance rows of the given focus rows: (libm oracle, engine arithmetic on the host),
    computed on all host threads (the C helpers release the GIL)."""
    pb = O.Problem(np.zeros((len(coords), 1)), np.zeros(len(coords)), coords, geographic=True, threads=1)
    row = gc_host.rows(coords)
    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        libm = list(ex.map(pb.distance_row, rows))
        cr = list(ex.map(row, rows))
    return libm, cr


def check_geo_thresholds(got, libm_rows, cr_rows, bw):
    """got[k] is the engine's threshold of the row whose distances are
    libm_rows[k] / cr_rows[k].  Returns (thresholds that differ from libm's,
    rows whose neighbour sets differ by near-ties)."""
    got = np.asarray(got)
    want_cr = np.array([O.adaptive_threshold(d, bw) for d in cr_rows])
    assert np.array_equal(got, want_cr), (bw, np.flatnonzero(got != want_cr)[:10])
    want = np.array([O.adaptive_threshold(d, bw) for d in libm_rows])
    differ = got != want
    assert differ.sum() <= max(1, GEO_THR_FRAC * len(got)), (bw, int(differ.sum()))
    assert ulps(got, want).max() <= GEO_THR_ULP, (bw, int(ulps(got, want).max()))
    near_ties = 0
    for k in range(len(got)):
        swapped = np.setxor1d(np.flatnonzero(libm_rows[k] < want[k]), np.flatnonzero(cr_rows[k] < got[k]))
        if len(swapped):
            near_ties += 1
            assert ulps(libm_rows[k][swapped], want[k]).max() <= GEO_THR_ULP, (bw, k, swapped)
    return int(differ.sum()), near_ties
