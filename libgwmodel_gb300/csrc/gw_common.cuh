// gw_common.cuh -- device-side types shared by the GWR kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gw_arith.h"

namespace gwgpu {

constexpr int kMaxP = 32;        // columns of X handled by the warp-per-location solve
constexpr int kTile = 16;        // points per data tile (skip granularity, Hilbert order)
constexpr int kRowBlock = 64;    // focus rows per contraction CTA

// Point coordinates in Hilbert order, structure of arrays.  Planar: u = x,
// v = y.  Geographic: u = longitude, v = latitude in degrees and uR/vR the
// same in radians, rounded as the reference rounds lon * (M_PI / 180).
struct DevPoints {
    int n;
    const double* u;
    const double* v;
    const double* uR;
    const double* vR;
    // geographic only, optional (null: absent): FP64 unit vectors (cos lat cos lon,
    // cos lat sin lon, sin lat) as three arrays of n, for the chord form of the distance
    const double* e;
};

// Axis-aligned bounds of one data tile of kTile consecutive (Hilbert-ordered) points.
struct TileBox {
    double ulo, uhi, vlo, vhi;
};

// Geographic tile bound: centre c of the tile's unit vectors (geodetic
// latitude on the unit sphere, the sphere of the haversine term S of the
// reference formula) and the largest 3-D chord rho from c to a member point.
struct TileCap {
    double cx, cy, cz, rho;
};

#if defined(__CUDACC__)
// Distance from focus point f to data point d, CRSDistance::distance
// (CRSDistance.cpp:122-131): planar EuclideanDistance(data - focus) or
// SpGcdist(data lon, focus lon, data lat, focus lat), the reference's double
// (correctly rounded sin/cos/atan for great-circle distances).
template <bool GEO>
__device__ __forceinline__ double pair_dist(const DevPoints& P, int d, double fu, double fv, double fuR,
                                            double fvR)
{
    if constexpr (GEO)
        return gw_gc_dist(P.u[d], fu, P.v[d], fv, P.uR[d], fuR, P.vR[d], fvR);
    else
        return gw_planar_dist(P.u[d], P.v[d], fu, fv);
}

// The reference's great-circle formula (CRSDistance.cpp:15-69) from FP64 unit
// vectors e = (cos lat cos lon, cos lat sin lon, sin lat): its haversine terms
// are S = sin^2 G cos^2 L + cos^2 F sin^2 L = |e_i - e_j|^2 / 4 and
// C = |e_i + e_j|^2 / 4, and sin F cos G = (sin lat_i + sin lat_j) / 2,
// cos F sin G = (sin lat_i - sin lat_j) / 2.  One square root, two divisions
// and one arctangent instead of three sine-cosine pairs, a square root and four
// divisions.  The chord of two nearby points carries an absolute error of a
// few 1e-16, i.e. ~1e-12 km in D: nothing against a bandwidth; the relative
// error elsewhere is a few ulp (CUDA's atan, within 2 ulp).
__device__ __forceinline__ double gc_dist_vec(double xi, double yi, double zi, double xj, double yj, double zj)
{
    const double a = 6378.137, f = 1.0 / 298.257223563;
    const double dx = xi - xj, dy = yi - yj, dz = zi - zj;
    const double sx = xi + xj, sy = yi + yj, sz = zi + zj;
    const double S = 0.25 * fma(dx, dx, fma(dy, dy, dz * dz));
    const double C = 0.25 * fma(sx, sx, fma(sy, sy, sz * sz));
    if (!(S > 0.0)) return 0.0;
    const double sc = S * C;
    const double rsc = sqrt(sc);
    const double inv = 1.0 / sc;             // 1/C = S inv, 1/S = C inv
    const double w = atan(rsc * (S * inv));  // atan(sqrt(S / C))
    const double R = rsc / w;
    const double D = 2.0 * w * a;
    const double H1 = (3.0 * R - 1.0) * (0.5 * S * inv);
    const double H2 = (3.0 * R + 1.0) * (0.5 * C * inv);
    const double sFcG = 0.5 * sz, cFsG = 0.5 * dz;
    return D * (1.0 + f * H1 * (sFcG * sFcG) - f * H2 * (cFsG * cFsG));
}

// Monotone map of a double onto uint64 (total order for non-NaN values).
__device__ __forceinline__ uint64_t dkey(double d)
{
    uint64_t b = (uint64_t)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// dkey((double)f) for f >= +0 (or +inf) from the bits of the float, in
// integer arithmetic only: a normal float's double pattern is
// (bits(f) + (896 << 23)) << 29 (exponent rebias 1023 - 127 = 896); a
// subnormal m 2^-149 with top bit s becomes exponent s + 874 and mantissa
// m << (52 - s).  Every case is a select, so no FP64 instruction is issued.
__device__ __forceinline__ uint64_t dkey_f(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint64_t normal = ((uint64_t)b + (896ull << 23)) << 29;
    const int s = 31 - __clz(b | 1u);
    const uint64_t sub = ((uint64_t)(s + 874) << 52) | (((uint64_t)b << (52 - s)) & 0x000fffffffffffffull);
    uint64_t bits = b >= 0x00800000u ? normal : (b == 0u ? 0ull : sub);
    bits = b >= 0x7f800000u ? (0x7ff0000000000000ull | ((uint64_t)(b & 0x7fffffu) << 29)) : bits;
    return bits | 0x8000000000000000ull;
}

__device__ __forceinline__ double keyd(uint64_t k)
{
    uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// Lower bound of the planar distance between two boxes (exact min over the
// boxes, evaluated with the same rounding as the point distance).
__device__ __forceinline__ double box_lower_bound(const TileBox& a, const TileBox& b)
{
    double dx = fmax(0.0, fmax(b.ulo - a.uhi, a.ulo - b.uhi));
    double dy = fmax(0.0, fmax(b.vlo - a.vhi, a.vlo - b.vhi));
    return sqrt(dx * dx + dy * dy);
}
// Lower bound (km) of the reference's ellipsoidal distance between any point
// of cap a and any point of cap b; 0 when no bound is proven.
//  * chord(P, Q) >= |ca - cb| - rho_a - rho_b (triangle inequality in R^3);
//  * S = chord^2 / 4 = sin^2(w), w the half central angle;
//  * D = 2 a w (1 + f (H1 sin^2F cos^2G - H2 cos^2F sin^2G)) with
//    H2 cos^2F sin^2G <= (3R + 1) / 2 <= 2 (since cos^2F sin^2G <= S) and
//    H1 >= -0.6 for w <= 1.2 rad, so D >= 2 a w (1 - 2.6 f) there.
__device__ __forceinline__ double cap_lower_bound(const TileCap& a, const TileCap& b)
{
    const double dx = a.cx - b.cx, dy = a.cy - b.cy, dz = a.cz - b.cz;
    const double cc = sqrt(dx * dx + dy * dy + dz * dz);
    const double lo = cc - a.rho - b.rho;
    if (!(lo > 0.0)) return 0.0;
    if (cc + a.rho + b.rho >= 1.8640781719344526) return 0.0;  // 2 sin(1.2)
    const double w = asin(0.5 * lo);
    return 2.0 * 6378.137 * w * (1.0 - 2.6 / 298.257223563);
}

// Cap covering caps[first..last].
__device__ __forceinline__ TileCap cap_union(const TileCap* caps, int first, int last)
{
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int q = first; q <= last; q++) {
        sx += caps[q].cx;
        sy += caps[q].cy;
        sz += caps[q].cz;
    }
    const double nrm = sqrt(sx * sx + sy * sy + sz * sz);
    TileCap u{sx / nrm, sy / nrm, sz / nrm, 0.0};
    for (int q = first; q <= last; q++) {
        const double dx = caps[q].cx - u.cx, dy = caps[q].cy - u.cy, dz = caps[q].cz - u.cz;
        u.rho = fmax(u.rho, sqrt(dx * dx + dy * dy + dz * dz) + caps[q].rho);
    }
    u.rho = u.rho * (1.0 + 1e-12) + 1e-15;
    return u;
}
// ---- FP32 tile tests (conservative, margins cover FP32 rounding) ----------
// Tile bound as float4: planar box (ulo, uhi, vlo, vhi) relative to the
// coordinate centroid, or geographic cap (cx, cy, cz, rho) on the unit sphere.

// Union of tile bounds tb[first..last].
template <bool GEO>
__device__ __forceinline__ float4 tb_union(const float4* tb, int first, int last)
{
    if (!GEO) {
        float4 b = tb[first];
        for (int q = first + 1; q <= last; q++) {
            const float4 c = tb[q];
            b.x = fminf(b.x, c.x); b.y = fmaxf(b.y, c.y);
            b.z = fminf(b.z, c.z); b.w = fmaxf(b.w, c.w);
        }
        return b;
    }
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int q = first; q <= last; q++) {
        sx += tb[q].x;
        sy += tb[q].y;
        sz += tb[q].z;
    }
    const float nrm = sqrtf(sx * sx + sy * sy + sz * sz);
    float4 u = make_float4(sx / nrm, sy / nrm, sz / nrm, 0.f);
    for (int q = first; q <= last; q++) {
        const float dx = tb[q].x - u.x, dy = tb[q].y - u.y, dz = tb[q].z - u.z;
        u.w = fmaxf(u.w, sqrtf(dx * dx + dy * dy + dz * dz) + tb[q].w);
    }
    u.w = u.w * (1.0f + 1e-5f) + 1e-6f;
    return u;
}

// Threshold of the far test for a largest bandwidth rmax (distance units):
// planar: squared distance; geographic: 3-D chord.  Returns -1 when no tile
// may be skipped.
template <bool GEO>
__device__ __forceinline__ float tb_far_threshold(double rmax)
{
    if (!(rmax > 0.0)) return -1.0f;
    if (!GEO) return (float)(rmax * rmax * (1.0 + 1e-4));
    const double w = rmax / (2.0 * 6378.137 * (1.0 - 2.6 / 298.257223563));
    if (w >= 1.2) return -1.0f;
    return (float)(2.0 * sin(w) * (1.0 + 1e-4));
}

// True when every pair between the focus bound fb and tile bound tb is at
// least as far as the threshold (so every weight of a compact kernel is 0).
template <bool GEO>
__device__ __forceinline__ bool tb_far(const float4& fb, const float4& tb, float thr)
{
    if (thr < 0.0f) return false;
    if (!GEO) {
        const float dx = fmaxf(0.0f, fmaxf(tb.x - fb.y, fb.x - tb.y));
        const float dy = fmaxf(0.0f, fmaxf(tb.z - fb.w, fb.z - tb.w));
        return fmaf(dx, dx, dy * dy) * (1.0f - 1e-5f) >= thr;
    }
    const float dx = tb.x - fb.x, dy = tb.y - fb.y, dz = tb.z - fb.z;
    const float cc = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    const float lo = (cc - fb.w - tb.w) * (1.0f - 1e-5f) - 1e-7f;
    const float hi = (cc + fb.w + tb.w) * (1.0f + 1e-5f) + 1e-7f;
    return lo >= thr && hi < 1.8640781f;
}
#endif  // __CUDACC__

}  // namespace gwgpu
