// mixed_weight.cuh -- FP32 distance and kernel weight of the mixed-precision
// path, shared by the tensor-core contraction and the refinement residual so
// both see the same weights.
#pragma once

#include "gw_common.cuh"

namespace gwgpu {

__device__ __forceinline__ float sin_poly(float x)
{
    // Taylor series to x^13, |x| <= pi/2
    float z = x * x;
    float p = -1.6059043836821614e-10f;        // -1/13!
    p = fmaf(p, z, 2.505210838544172e-08f);    //  1/11!
    p = fmaf(p, z, -2.7557319223985893e-06f);  // -1/9!
    p = fmaf(p, z, 1.984126984126984e-04f);    //  1/7!
    p = fmaf(p, z, -8.333333333333333e-03f);   // -1/5!  (sign alternates: x - x^3/6 + ...)
    p = fmaf(p, z, 1.6666666666666666e-01f);   //  1/3!
    return x - x * z * p;
}

// asin(x) / x for S = x^2 <= 0.25, from the Maclaurin series
// asin x = sum_k (2k)! / (4^k (k!)^2 (2k + 1)) x^(2k+1) truncated after k = 10
// (the first omitted term is below 2e-9 relative at S = 0.25).
__device__ __forceinline__ float asin_over_x(float S)
{
    float p = 8.3903358096168155e-03f;      // k = 10: 46189 / 5505024
    p = fmaf(p, S, 9.7616095291940789e-03f);  // k = 9: 12155 / 1245184
    p = fmaf(p, S, 1.1551800896139706e-02f);  // k = 8: 6435 / 557056
    p = fmaf(p, S, 1.3964843750000000e-02f);  // k = 7: 143 / 10240
    p = fmaf(p, S, 1.7352764423076924e-02f);  // k = 6: 231 / 13312
    p = fmaf(p, S, 2.2372159090909092e-02f);  // k = 5: 63 / 2816
    p = fmaf(p, S, 3.0381944444444444e-02f);  // k = 4: 35 / 1152
    p = fmaf(p, S, 4.4642857142857144e-02f);  // k = 3: 5 / 112
    p = fmaf(p, S, 7.5000000000000000e-02f);  // k = 2: 3 / 40
    p = fmaf(p, S, 1.6666666666666666e-01f);  // k = 1: 1 / 6
    return fmaf(p, S, 1.0f);
}

// Haversine term S = sin^2(theta / 2) of the pair: a quarter of the squared
// chord between the hi/lo unit vectors.
__device__ __forceinline__ float geo_haversine32(const float4& fa, const float4& fb, const float4& pa, const float4& pb)
{
    const float dx = (pa.x - fa.x) + (pb.x - fb.x);
    const float dy = (pa.y - fa.y) + (pb.y - fb.y);
    const float dz = (pa.z - fa.z) + (pb.z - fb.z);
    return 0.25f * fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// FP32 great-circle distance (km) of the reference's Lambert formula, given
// the haversine term S of the pair.  With S = sin^2 w (w = theta / 2) and
// C = 1 - S: w = sqrt(S) asin_over_x(S) and R = sqrt(S C) / w =
// sqrt(C) / asin_over_x(S) for S <= 0.25; atan2 beyond.
__device__ __forceinline__ float geo_dist32_from_S(float S, const float4& fa, const float4& fb, const float4& fc,
                                                   const float4& pa, const float4& pb, const float4& pc)
{
    if (!(S > 0.0f)) return 0.0f;
    const float C = fmaxf(1.0f - S, 0.0f);
    float w, R;
    if (S <= 0.25f) {
        const float P = asin_over_x(S);
        w = S * rsqrtf(S) * P;
        R = __fdividef(C * rsqrtf(C), P);
    } else {
        const float sq = sqrtf(S), cq = sqrtf(C);
        w = atan2f(sq, cq);
        R = __fdividef(sq * cq, w);
    }
    const float dlat = (pa.w - fa.w) + (pb.w - fb.w);            // degrees
    const float G = dlat * 8.7266462599716478846e-3f;            // (pi/180)/2
    const float sG = sin_poly(G);
    const float sG2 = sG * sG, cG2 = 1.0f - sG2;
    const float sF = pc.x * fc.y + pc.y * fc.x;                  // sin((lat_a+lat_b)/2)
    const float cF = pc.y * fc.y - pc.x * fc.x;
    const float sF2 = sF * sF, cF2 = cF * cF;
    const float H1 = __fdividef(3.0f * R - 1.0f, 2.0f * C);
    const float H2 = __fdividef(3.0f * R + 1.0f, 2.0f * S);
    const float f = 1.0f / 298.257223563f;
    return 2.0f * 6378.137f * w * (1.0f + f * H1 * sF2 * cG2 - f * H2 * cF2 * sG2);
}

// FP32 great-circle distance (km) of the reference's Lambert formula with the
// haversine term taken from the 3-D chord of hi/lo unit vectors.
__device__ __forceinline__ float geo_dist32(const float4& fa, const float4& fb, const float4& fc, const float4& pa,
                                            const float4& pb, const float4& pc)
{
    return geo_dist32_from_S(geo_haversine32(fa, fb, pa, pb), fa, fb, fc, pa, pb, pc);
}

// Haversine cut-off of a focus row for a compactly supported kernel with
// threshold r (km): a pair with S above it lies beyond r, so its weight is 0.
// The Lambert distance satisfies D >= 2 a w (1 - 2.6 f) for w <= 1.2 rad and
// w >= sin w = sqrt(S); the 1e-3 margin is far above the FP32 rounding of S
// and D, so the cut never drops a pair whose computed weight is nonzero.
// Returns +inf (no cut) where the bound does not apply.
__device__ __forceinline__ float geo_s_cut(float r)
{
    const float x = r * (1.0f + 1e-3f) / (2.0f * 6378.137f * (1.0f - 2.6f / 298.257223563f));
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

// Weight of data point j (coordinates at pts) for a focus point with the
// given FP32 data, threshold r and 1/r^2 -- exactly what the contraction uses.
template <bool GEO>
__device__ __forceinline__ float mixed_weight(const float4* __restrict__ pts, int j, const float4& fa,
                                              const float4& fb, const float4& fc, int kernel, float r, float inv_r2)
{
    float d2;
    if (GEO) {
        float d = geo_dist32(fa, fb, fc, pts[3 * (size_t)j], pts[3 * (size_t)j + 1], pts[3 * (size_t)j + 2]);
        d2 = d * d;
    } else {
        d2 = planar_d2_32(fa, pts[j]);
    }
    return weight32(kernel, d2, r, inv_r2);
}

}  // namespace gwgpu
