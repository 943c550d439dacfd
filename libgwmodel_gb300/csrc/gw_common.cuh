// gw_common.cuh -- device-side types shared by the GWR kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gw_arith.h"

namespace gwgpu {

constexpr int kMaxP = 32;        // columns of X handled by the warp-per-location solve
constexpr int kTile = 16;        // points per data tile (skip granularity, Morton order)
constexpr int kRowBlock = 64;    // focus rows per contraction CTA

// Point coordinates in Morton order, structure of arrays.  Planar: u = x,
// v = y.  Geographic: u = longitude, v = latitude in degrees and uR/vR the
// same in radians, rounded as the reference rounds lon * (M_PI / 180).
struct DevPoints {
    int n;
    const double* u;
    const double* v;
    const double* uR;
    const double* vR;
};

// Axis-aligned bounds of one data tile of kTile consecutive (Morton) points.
struct TileBox {
    double ulo, uhi, vlo, vhi;
};

#if defined(__CUDACC__)
// Distance from focus point f to data point d, CRSDistance::distance
// (CRSDistance.cpp:122-131): planar EuclideanDistance(data - focus) or
// SpGcdist(data lon, focus lon, data lat, focus lat).
template <bool GEO>
__device__ __forceinline__ double pair_dist(const DevPoints& P, int d, double fu, double fv, double fuR,
                                            double fvR)
{
    if constexpr (GEO)
        return gw_gc_dist(P.u[d], fu, P.v[d], fv, P.uR[d], fuR, P.vR[d], fvR);
    else
        return gw_planar_dist(P.u[d], P.v[d], fu, fv);
}

// Monotone map of a double onto uint64 (total order for non-NaN values).
__device__ __forceinline__ uint64_t dkey(double d)
{
    uint64_t b = (uint64_t)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
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
#endif  // __CUDACC__

}  // namespace gwgpu
