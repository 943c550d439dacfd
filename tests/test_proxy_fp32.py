"""The mixed path's FP32 great-circle proxy (mixed_weight.cuh: geo_chord32,
geo_d2_near, geo_d2_far), restated in numpy float32 arithmetic on the CPU,
against the reference's FP64 formula (the oracle's SpGcdist,
CRSDistance.cpp:15-69).

The exact select trusts the proxy within a band of 2^-16 relative (plus 1e-6
km) for pairs below 15,000 km, and the distance cache relies on the proxy
being symmetric bit for bit.  This restatement rounds every operation to FP32
as the kernels do (an FMA as one rounding of the exact product-sum); it uses
a correctly rounded reciprocal square root and reciprocal where the kernels
use the hardware approximations (a few ulp more), so its bar sits far below
the band: 2e-6 relative."""
import numpy as np
import pytest

import oracle as O

F32 = np.float32
A_KM = 6378.137
K4 = F32(4.0 * A_KM * A_KM)
FLAT = F32(1.0 / 298.257223563)
ASIN_C = [4.2417373813264260e-02, 2.3993999622970812e-02, 4.5520635638035500e-02, 7.4946966873681580e-02,
          1.6666782005777223e-01, 9.9999999598373800e-01]


def fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(F32)


def rsqrt(x):
    with np.errstate(divide="ignore", invalid="ignore"):
        return (1.0 / np.sqrt(np.asarray(x, np.float64))).astype(F32)


def rcp(x):
    with np.errstate(divide="ignore"):
        return (1.0 / np.asarray(x, np.float64)).astype(F32)


def asin_over_x(s):
    p = np.full_like(s, F32(ASIN_C[0]))
    for c in ASIN_C[1:]:
        p = fma(p, s, F32(c))
    return p


def records(lon_deg, lat_deg):
    lon, lat = np.radians(lon_deg), np.radians(lat_deg)
    e = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])
    hi = e.astype(F32)
    return hi, (e - hi).astype(F32)


def proxy_d2(fh, fl, ph, pl):
    """Squared distance (km^2) of focus records (fh, fl) and point records (ph, pl)."""
    d = [((ph[k] - fh[k]) + (pl[k] - fl[k])).astype(F32) for k in range(3)]
    s = (F32(0.25) * fma(d[0], d[0], fma(d[1], d[1], (d[2] * d[2]).astype(F32)))).astype(F32)
    dz = d[2]
    zs = ((ph[2] + fh[2]) + (pl[2] + fl[2])).astype(F32)
    near = s <= F32(0.25)
    sm = [((ph[k] + fh[k]) + (pl[k] + fl[k])).astype(F32) for k in range(3)]
    cf = (F32(0.25) * fma(sm[0], sm[0], fma(sm[1], sm[1], (sm[2] * sm[2]).astype(F32)))).astype(F32)
    c = np.where(near, np.maximum(F32(1.0) - s, F32(0.0)), cf).astype(F32)
    with np.errstate(invalid="ignore"):
        cq = np.where(c > 0, (c * rsqrt(c)).astype(F32), F32(0.0))
        rs = rsqrt(s)
        y = (c * rcp(fma(F32(2.0), (s * rs).astype(F32), F32(2.0)))).astype(F32)
        z = np.where(near, s, y).astype(F32)
        pz = asin_over_x(z)
        zr = np.where(z > 0, (z * rsqrt(z)).astype(F32), F32(0.0))
        far_w = fma((F32(-2.0) * zr).astype(F32), pz, F32(1.5707963267948966))
        a = np.where(near, pz, (far_w * rs).astype(F32)).astype(F32)
    t1, t2 = fma(F32(3.0), cq, -a), fma(F32(3.0), cq, a)
    num = fma((t1 * (zs * zs).astype(F32)).astype(F32), s, (-((t2 * (dz * dz).astype(F32)).astype(F32)) * c).astype(F32))
    q = fma((F32(0.125) * FLAT * num).astype(F32), rcp(np.maximum((s * c).astype(F32), F32(1e-30))), a)
    return (K4 * s * (q * q).astype(F32)).astype(F32)


def exact(lon1, lon2, lat1, lat2):
    return np.array([O.gcdist(a, b, c, d) for a, b, c, d in zip(lon1, lon2, lat1, lat2)])


def test_symmetric_bit_for_bit():
    rng = np.random.default_rng(21)
    n = 20000
    lon = rng.uniform(-180.0, 180.0, (2, n))
    lat = np.degrees(np.arcsin(rng.uniform(-1.0, 1.0, (2, n))))
    ah, al = records(lon[0], lat[0])
    bh, bl = records(lon[1], lat[1])
    np.testing.assert_array_equal(proxy_d2(ah, al, bh, bl), proxy_d2(bh, bl, ah, al))


@pytest.mark.parametrize("region", ["config2", "sphere"])
def test_relative_error_below_the_band(region):
    rng = np.random.default_rng(22)
    n = 3000
    if region == "config2":
        lon = rng.uniform(-10.0, 30.0, (2, n))
        lat = rng.uniform(35.0, 60.0, (2, n))
    else:
        lon = rng.uniform(-180.0, 180.0, (2, n))
        lat = np.degrees(np.arcsin(rng.uniform(-0.999, 0.999, (2, n))))
    ah, al = records(lon[0], lat[0])
    bh, bl = records(lon[1], lat[1])
    d32 = np.sqrt(proxy_d2(ah, al, bh, bl).astype(np.float64))
    ref = exact(lon[0], lon[1], lat[0], lat[1])
    keep = (ref > 1e-3) & (ref < 15000.0)
    err = np.abs(d32[keep] - ref[keep]) / ref[keep]
    assert err.max() < 2e-6, err.max()


@pytest.mark.parametrize("delta", [1e-2, 1e-4, 1e-6])
def test_near_the_antipode(delta):
    """Within delta rad of the antipode, where 1 - S and (1 - sqrt S) / 2 would
    lose their precision (the earlier form returned 0 within 1e-4 rad)."""
    rng = np.random.default_rng(23)
    n = 3000
    lon1 = rng.uniform(-180.0, 180.0, n)
    lat1 = np.degrees(np.arcsin(rng.uniform(-0.99, 0.99, n)))
    ang = rng.uniform(0.0, 2.0 * np.pi, n)
    lon2 = (lon1 + 180.0 + np.degrees(delta * np.cos(ang) / np.cos(np.radians(lat1))) + 180.0) % 360.0 - 180.0
    lat2 = -lat1 + np.degrees(delta * np.sin(ang))
    ah, al = records(lon1, lat1)
    bh, bl = records(lon2, lat2)
    d32 = np.sqrt(proxy_d2(ah, al, bh, bl).astype(np.float64))
    ref = exact(lon1, lon2, lat1, lat2)
    err = np.abs(d32 - ref) / ref
    assert err.max() < 2e-6, err.max()
