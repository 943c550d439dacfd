"""Distance cache of the mixed geographic contraction.

The cache holds the FP32 squared great-circle distance of every pair, filled
with the weight producer's own arithmetic, so an engine that reads it must
give bit-identical criteria, coefficients and diagnostics to one that
recomputes the distances.  The data below spread over the whole sphere, so
both the near-angle and the far-angle forms of the distance occur, and n is
not a multiple of the 128-row block or the 32-point tile."""
import numpy as np
import pytest

from libgwmodel_gb300 import Engine

pytestmark = pytest.mark.gpu


def sphere_problem(n, p, seed):
    rng = np.random.default_rng(seed)
    lon = rng.uniform(-180.0, 180.0, n)
    lat = np.degrees(np.arcsin(rng.uniform(-0.95, 0.95, n)))
    coords = np.column_stack([lon, lat])
    x = np.column_stack([np.ones(n)] + [rng.standard_normal(n) for _ in range(p - 1)])
    beta = 1.0 + 0.5 * np.sin(np.radians(lat))[:, None] * rng.uniform(-1, 1, p)[None, :]
    y = (x * beta).sum(axis=1) + 0.3 * rng.standard_normal(n)
    return x, y, coords


def engines(x, y, coords):
    out = []
    for limit in (-1, 0):
        e = Engine(0)
        e.set_data(x, y, coords, True)
        e.set_precision(1)
        e.set_distance_cache(limit)
        out.append(e)
    return out


@pytest.mark.parametrize("kernel,adaptive,bws", [(2, True, [25, 300, 2000]), (0, True, [40, 700]),
                                                 (2, False, [1500.0, 6000.0]), (0, False, [800.0])])
@pytest.mark.parametrize("crit", [0, 1])
def test_cached_criterion_bit_identical(kernel, adaptive, bws, crit):
    x, y, coords = sphere_problem(2345, 5, 11)
    cached, plain = engines(x, y, coords)
    for bw in bws:
        a = cached.criterion(bw, adaptive, kernel, crit)
        b = plain.criterion(bw, adaptive, kernel, crit)
        assert a == b, (bw, a, b)
    assert cached.distance_cache_active()
    assert not plain.distance_cache_active()


@pytest.mark.parametrize("n,bws", [(2345, [2, 25, 300, 1000, 2344]), (25003, [21000, 4000, 60])])
def test_cached_thresholds_bit_identical(n, bws):
    """The selects of the cached engine read the proxy distances from the
    cache (both select widths: ranks above 20,000 take the four-warp form)."""
    x, y, coords = sphere_problem(n, 3, 15)
    cached, plain = engines(x, y, coords)
    for bw in bws:
        np.testing.assert_array_equal(cached.thresholds(bw), plain.thresholds(bw), err_msg=str(bw))
    assert cached.distance_cache_active()


def test_cached_fit_bit_identical():
    x, y, coords = sphere_problem(3001, 6, 12)
    cached, plain = engines(x, y, coords)
    fa = cached.fit(120, True, 2, store_s=True)
    fb = plain.fit(120, True, 2, store_s=True)
    for u, v in zip(fa, fb):
        np.testing.assert_array_equal(np.asarray(u), np.asarray(v))


def test_cached_golden_search_bit_identical():
    x, y, coords = sphere_problem(1800, 4, 13)
    cached, plain = engines(x, y, coords)
    bw_a, crit_a = cached.golden(True, 2, 0, 20.0, 1800.0)[:2]
    bw_b, crit_b = plain.golden(True, 2, 0, 20.0, 1800.0)[:2]
    assert bw_a == bw_b
    assert np.array_equal(np.asarray(crit_a), np.asarray(crit_b))


def test_cache_fills_once_per_dataset_and_moves_between_engines():
    x, y, coords = sphere_problem(2000, 4, 14)
    a = Engine(0)
    a.set_data(x, y, coords, True)
    a.set_precision(1)
    a.enable_stats(True)
    for bw in (50, 400, 900):
        a.criterion(bw, True, 2, 0)
    assert a.stats()["d2c_fills"] == 1
    assert a.distance_cache_active()
    # a second engine takes the device's cache over; the first refills on its next use
    x2, y2, c2 = sphere_problem(2100, 4, 15)
    b = Engine(0)
    b.set_data(x2, y2, c2, True)
    b.set_precision(1)
    vb = b.criterion(300, True, 2, 0)
    assert b.distance_cache_active() and not a.distance_cache_active()
    va = a.criterion(400, True, 2, 0)
    assert a.stats()["d2c_fills"] == 2
    # clearing forgets the contents; releasing frees the buffer
    a.clear_cache()
    assert not a.distance_cache_active()
    a.release_distance_cache()
    ref_b = Engine(0)
    ref_b.set_data(x2, y2, c2, True)
    ref_b.set_precision(1)
    ref_b.set_distance_cache(0)
    assert vb == ref_b.criterion(300, True, 2, 0)
    ref_a = Engine(0)
    ref_a.set_data(x, y, coords, True)
    ref_a.set_precision(1)
    ref_a.set_distance_cache(0)
    assert va == ref_a.criterion(400, True, 2, 0)


def test_cache_off_for_planar_and_fp64():
    rng = np.random.default_rng(3)
    n = 1500
    coords = rng.uniform(0, 100, (n, 2))
    x = np.column_stack([np.ones(n), rng.standard_normal(n)])
    y = x @ np.array([1.0, 2.0]) + rng.standard_normal(n)
    e = Engine(0)
    e.set_data(x, y, coords, False)
    e.set_precision(1)
    e.criterion(100, True, 2, 0)
    assert not e.distance_cache_active()
    g = Engine(0)
    g.set_data(x, y, coords * 0.5, True)
    g.criterion(100, True, 2, 0)  # FP64 drop-in
    assert not g.distance_cache_active()


@pytest.mark.parametrize("geographic", [True, False])
def test_wide_x_keeps_shared_memory_weights(geographic):
    """p = 20 (Z 230 columns, npad 240 > 192): the contraction keeps its weight
    tiles in shared memory.  Cached and uncached agree bit for bit, and the
    mixed criterion stays within 1e-5 of the FP64 engine."""
    n, p = 1500, 20
    rng = np.random.default_rng(21)
    if geographic:
        x, y, coords = sphere_problem(n, p, 22)
        coords = np.column_stack([rng.uniform(-10, 30, n), rng.uniform(35, 60, n)])
    else:
        coords = rng.uniform(0, 100, (n, 2))
        x = np.column_stack([np.ones(n)] + [rng.standard_normal(n) for _ in range(p - 1)])
        y = x @ rng.uniform(-1, 1, p) + 0.3 * rng.standard_normal(n)
    cached, plain = engines(x, y, coords) if geographic else (None, None)
    e64 = Engine(0)
    e64.set_data(x, y, coords, geographic)
    emx = Engine(0)
    emx.set_data(x, y, coords, geographic)
    emx.set_precision(1)
    for bw in (120, 600):
        c64 = e64.criterion(bw, True, 2, 0)
        cmx = emx.criterion(bw, True, 2, 0)
        assert abs(cmx - c64) <= 1e-5 * abs(c64), (bw, cmx, c64)
        if geographic:
            assert cached.criterion(bw, True, 2, 0) == plain.criterion(bw, True, 2, 0)
