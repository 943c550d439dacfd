// mixed_weight.cuh -- FP32 distance and kernel weight of the mixed-precision
// path, shared by the tensor-core contraction and the refinement residual so
// both see the same weights.
#pragma once

#include "gw_common.cuh"

namespace gwgpu {

// Point records of the mixed path.  Geographic: the unit vector of the point
// split into FP32 hi + lo, as two float4 (x_hi, y_hi, z_hi, 0), (x_lo, y_lo,
// z_lo, 0), so z = sin(lat).  Planar: one float4 (u_hi, u_lo, v_hi, v_lo)
// relative to the centroid.

// The hardware approximations of 1/sqrt(x) and 1/x with subnormal inputs and
// results flushed to zero.  The proxy arithmetic never meets a subnormal (its
// smallest nonzero intermediate values are near 1e-31), so the flush costs no
// precision and saves the subnormal handling; every proxy value of every
// kernel is computed with these, so all kernels see the same values.
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float rcp_ftz(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// asin(x) / x as a polynomial in S = x^2 on [0, 0.25]: the degree-5 Chebyshev
// interpolant at the Chebyshev nodes of that interval, converted to monomials
// (largest relative deviation 4.8e-9, below FP32 rounding).
__device__ __forceinline__ float asin_over_x(float S)
{
    float p = 4.2417373813264260e-02f;
    p = fmaf(p, S, 2.3993999622970812e-02f);
    p = fmaf(p, S, 4.5520635638035500e-02f);
    p = fmaf(p, S, 7.4946966873681580e-02f);
    p = fmaf(p, S, 1.6666782005777223e-01f);
    return fmaf(p, S, 9.9999999598373800e-01f);
}

constexpr float kGeoA = 6378.137f;                  // WGS-84 semi-major axis (km)
constexpr float kGeoF = 1.0f / 298.257223563f;      // WGS-84 flattening
constexpr float kGeoK = 4.0f * kGeoA * kGeoA;       // (2a)^2

// Chord terms of a pair of geographic records: S = sin^2 w = |chord|^2 / 4
// (w = half the central angle), dz = sin phi_p - sin phi_f and
// zs = sin phi_p + sin phi_f, each from the hi and lo parts separately.
// Swapping the focus and the point negates every difference exactly and
// leaves every sum unchanged, so every value below is the same for (f, p)
// and (p, f): the distance of a pair is symmetric bit for bit.
struct GeoChord {
    float S, dz, zs;
};

__device__ __forceinline__ GeoChord geo_chord32(const float4& fa, const float4& fb, const float4& pa, const float4& pb)
{
    const float dx = (pa.x - fa.x) + (pb.x - fb.x);
    const float dy = (pa.y - fa.y) + (pb.y - fb.y);
    const float dz = (pa.z - fa.z) + (pb.z - fb.z);
    GeoChord g;
    g.S = 0.25f * fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    g.dz = dz;
    g.zs = (pa.z + fa.z) + (pb.z + fb.z);
    return g;
}

// Squared great-circle distance (km^2) of the reference's Lambert formula
// (CRSDistance.cpp:15-81) in FP32, given A = w / sqrt(S).  With latitudes phi:
//   sin^2F cos^2G = ((sin phi_a + sin phi_b) / 2)^2  and
//   cos^2F sin^2G = ((sin phi_a - sin phi_b) / 2)^2,
// so with R = sqrt(S C) / w = sqrt(C) / A (C = 1 - S) the formula
// D = 2 a w (1 + f (H1 sin^2F cos^2G - H2 cos^2F sin^2G)), H1 = (3R - 1)/(2C),
// H2 = (3R + 1)/(2S), becomes D^2 = (2a)^2 S Q^2 with Q = A (1 + c),
//   c = (f / 8) [(3 sqrt C - A) zs^2 S - (3 sqrt C + A) dz^2 C] / (A S C),
// so Q = A + (f / 8) num / (S C): A cancels from the correction.  num is
// O(S) (|dz| <= 2 sqrt S), so clamping S C below at 1e-30 only keeps the
// reciprocal finite: S = 0 gives Q = A and D = 0.  Towards the antipode num is
// O(C) (zs^2 <= 4 C), so the correction stays bounded given accurate C and zs.
// Here cq = sqrt(C).
__device__ __forceinline__ float geo_lambert_d2(const GeoChord& g, float A, float C, float cq)
{
    const float S = g.S;
    const float t1 = fmaf(3.0f, cq, -A), t2 = fmaf(3.0f, cq, A);
    const float num = fmaf(t1 * (g.zs * g.zs), S, -(t2 * (g.dz * g.dz)) * C);
    const float Q = fmaf((0.125f * kGeoF) * num, rcp_ftz(fmaxf(S * C, 1e-30f)), A);
    return kGeoK * S * (Q * Q);
}

// Half angles up to 60 degrees (S <= 0.25): A from the polynomial directly and
// C = 1 - S (at least 0.75: no precision lost).  The caller makes sure S <= 0.25.
__device__ __forceinline__ float geo_d2_near(const GeoChord& g)
{
    const float C = fmaxf(1.0f - g.S, 0.0f);
    return geo_lambert_d2(g, asin_over_x(g.S), C, C * rsqrt_ftz(C));
}

// Any S, from the chord terms g of the focus record (fa, fb) and the point
// record (pa, pb).  Beyond S = 0.25 C = cos^2 w = |f + p|^2 / 4 comes from the
// sum of the two unit vectors (hi + lo), which keeps its relative precision
// towards the antipode where 1 - S loses it, and
// asin x = pi/2 - 2 asin(sqrt y) with y = (1 - sqrt S) / 2 = C / (2 (1 + sqrt S))
// <= 0.25 reuses the polynomial.  Branch-free (the cases are selects), and
// equal to geo_d2_near wherever S <= 0.25.
__device__ __forceinline__ float geo_d2_far(const GeoChord& g, const float4& fa, const float4& fb, const float4& pa,
                                            const float4& pb)
{
    const float S = g.S;
    const bool near = S <= 0.25f;
    const float sx = (pa.x + fa.x) + (pb.x + fb.x);
    const float sy = (pa.y + fa.y) + (pb.y + fb.y);
    const float sz = g.zs;  // sin phi_p + sin phi_f
    const float C = near ? fmaxf(1.0f - S, 0.0f) : 0.25f * fmaf(sx, sx, fmaf(sy, sy, sz * sz));
    const float cq = C > 0.0f ? C * rsqrt_ftz(C) : 0.0f;
    const float rs = rsqrt_ftz(S);
    const float y = C * rcp_ftz(fmaf(2.0f, S * rs, 2.0f));  // (1 - sqrt S) / 2
    const float z = near ? S : y;
    const float Pz = asin_over_x(z);
    const float zr = z > 0.0f ? z * rsqrt_ftz(z) : 0.0f;
    const float far_w = fmaf(-2.0f * zr, Pz, 1.5707963267948966f);  // asin(sqrt S)
    return geo_lambert_d2(g, near ? Pz : far_w * rs, C, cq);
}

__device__ __forceinline__ float geo_d2_32(const float4& fa, const float4& fb, const float4& pa, const float4& pb)
{
    return geo_d2_far(geo_chord32(fa, fb, pa, pb), fa, fb, pa, pb);
}

// True when a pair with haversine term S lies beyond a compact kernel's
// threshold whose cut-off (geo_s_cut) is s_cut.
__device__ __forceinline__ bool geo_beyond(float S, float s_cut) { return S >= s_cut && S <= 0.86f; }

// FP32 great-circle distance (km), the square root of geo_d2_32.
__device__ __forceinline__ float geo_dist32(const float4& fa, const float4& fb, const float4& pa, const float4& pb)
{
    const float d2 = geo_d2_32(fa, fb, pa, pb);
    return d2 > 0.0f ? d2 * rsqrt_ftz(d2) : 0.0f;
}

// Haversine cut-off of a focus row for a compactly supported kernel with
// threshold r (km): a pair with S above it lies beyond r, so its weight is 0.
// The Lambert distance satisfies D >= 2 a w (1 - 2.6 f) for w <= 1.2 rad and
// w >= sin w = sqrt(S); the 1e-3 margin is far above the FP32 rounding of S
// and D, so the cut never drops a pair whose computed weight is nonzero.
// Returns +inf (no cut) where the bound does not apply.
__device__ __forceinline__ float geo_s_cut(float r)
{
    const float x = r * (1.0f + 1e-3f) / (2.0f * kGeoA * (1.0f - 2.6f * kGeoF));
    const float s = x * x;
    return (r > 0.0f && s < 0.86f) ? s : __int_as_float(0x7f800000);
}

__device__ __forceinline__ float weight32(int kernel, float d2, float r, float inv_r2)
{
    switch (kernel) {
    case GW_KERNEL_GAUSSIAN:
        return __expf(-0.5f * d2 * inv_r2);
    case GW_KERNEL_EXPONENTIAL:
        return __expf(-sqrtf(d2) / r);
    case GW_KERNEL_BISQUARE: {
        float t = 1.0f - d2 * inv_r2;
        return d2 < r * r ? t * t : 0.0f;
    }
    case GW_KERNEL_TRICUBE: {
        float q = sqrtf(d2) / r;
        float t = 1.0f - q * q * q;
        return d2 < r * r ? t * t * t : 0.0f;
    }
    default:
        return d2 < r * r ? 1.0f : 0.0f;
    }
}


// Planar FP32 squared distance from hi/lo coordinates relative to the centroid.
__device__ __forceinline__ float planar_d2_32(const float4& f, const float4& p)
{
    const float dx = (p.x - f.x) + (p.y - f.y);
    const float dy = (p.z - f.z) + (p.w - f.w);
    return fmaf(dx, dx, dy * dy);
}

// Weight of data point j (record at pts) for a focus point with record (fa,
// fb), threshold r and 1/r^2 -- exactly what the contraction uses.
template <bool GEO>
__device__ __forceinline__ float mixed_weight(const float4* __restrict__ pts, int j, const float4& fa,
                                              const float4& fb, int kernel, float r, float inv_r2)
{
    const float d2 = GEO ? geo_d2_32(fa, fb, pts[2 * (size_t)j], pts[2 * (size_t)j + 1]) : planar_d2_32(fa, pts[j]);
    return weight32(kernel, d2, r, inv_r2);
}

}  // namespace gwgpu
