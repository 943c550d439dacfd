// k_contract64.cu -- FP64 fused distance -> kernel weight -> W.Z contraction.
//
// For every focus row i this produces G[i, :] = sum_j w_ij^wpow Z[j, :],
// where Z[j, :] holds the packed products x_j x_j^T and x_j y_j.  One pass
// therefore yields X^T W_i X and X^T W_i y for every location at once
// (GWRBasic.cpp:502-504 does two products per location against an explicit
// n-vector of weights).  The weight tile is computed in the producer stage
// from the coordinates and never written to memory.  Compactly supported
// kernels (bisquare, tricube, boxcar) skip data tiles whose box is farther
// than the largest threshold of the CTA's 64 rows (planar coordinates).
//
// GB300 runs FP64 at a small fraction of its FP32/tensor rate, so this
// kernel is bound by the FP64 pipe; its job is to be the exact drop-in.
#include "gw_common.cuh"
#include "gw_kernels.h"

namespace gwgpu {

namespace {

constexpr int CT_THREADS = 256;
constexpr int CT_BM = kRowBlock;  // 64 focus rows
constexpr int CT_BK = kTile;      // 16 data points per tile
constexpr int CT_ROWS_PER_THREAD = CT_BM / 16;

// w_ij in FP64.  Planar bisquare and gaussian weights depend on d^2 only, so
// they skip the square root and the divisions: with r2 = r^2 and ir2 = 1 / r^2
// per row they cost a handful of FP64 operations, which is what bounds this
// kernel on GB300.  They differ from the reference's sqrt-then-square form
// (BandwidthWeight.cpp:60-91) by an ulp or two of d^2; at d ~ r, where the two
// comparisons d < r and d^2 < r2 can disagree, the bisquare weight is
// (1 - d^2/r^2)^2 ~ 1e-32.  The boxcar weight is a unit step at exactly that
// point (an adaptive threshold is the distance of a data point), so it keeps
// the reference's d < r, as do the other kernels and geographic distances.
template <bool GEO>
__device__ __forceinline__ double pair_weight64(int kernel, double du, double dv, double duR, double dvR, double fu,
                                                double fv, double fuR, double fvR, double r, double r2, double ir2)
{
    if (!GEO && (kernel == GW_KERNEL_BISQUARE || kernel == GW_KERNEL_GAUSSIAN)) {
        const double dx = du - fu, dy = dv - fv;
        const double d2 = fma(dy, dy, dx * dx);
        if (kernel == GW_KERNEL_GAUSSIAN) return exp(d2 * (-0.5 * ir2));
        const double t = 1.0 - d2 * ir2;
        return d2 < r2 ? t * t : 0.0;
    }
    double d;
    if constexpr (GEO)
        d = kernel == GW_KERNEL_BOXCAR ? gw_gc_dist(du, fu, dv, fv, duR, fuR, dvR, fvR)
                                       : gw_gc_dist_fast(du, fu, dv, fv, duR, fuR, dvR, fvR);
    else
        d = gw_planar_dist(du, dv, fu, fv);
    return gw_kernel_weight(kernel, d, r);
}

// w_ij of a geographic pair from the unit vectors (bisquare, tricube, gaussian,
// exponential; the boxcar step at d = r keeps the reference formula).
__device__ __forceinline__ double pair_weight64_vec(int kernel, double xi, double yi, double zi, double xj, double yj,
                                                    double zj, double r, double ir2)
{
    const double d = gc_dist_vec(xi, yi, zi, xj, yj, zj);
    if (kernel == GW_KERNEL_BISQUARE) {
        const double t = 1.0 - d * d * ir2;
        return d < r ? t * t : 0.0;
    }
    if (kernel == GW_KERNEL_GAUSSIAN) return exp(d * d * (-0.5 * ir2));
    return gw_kernel_weight(kernel, d, r);
}

template <bool GEO, int NC>
__global__ void __launch_bounds__(CT_THREADS)
    k_contract64(DevPoints P, const float4* __restrict__ tb16, DevPoints F, const float4* __restrict__ ftb16,
                 const double* __restrict__ Z, int ldz, int mcols, double* __restrict__ G, int ldg,
                 const double* __restrict__ thr, double bw, int kernel, int exclude_self, int wpow, int skip_tiles)
{
    constexpr int NCOL = NC * 16;
    __shared__ double sW[CT_BM][CT_BK + 1];
    __shared__ double sZ[CT_BK][NCOL];
    __shared__ double sfu[CT_BM], sfv[CT_BM], sfuR[CT_BM], sfvR[CT_BM], sthr[CT_BM], sr2[CT_BM], sir2[CT_BM];
    __shared__ double sfe[3][CT_BM];
    __shared__ double sred[CT_THREADS / 32];
    __shared__ float4 sbound;

    const int n = P.n, nf = F.n;  // data points, focus rows (the data themselves, or prediction points)
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int row0 = blockIdx.x * CT_BM;
    // unit-vector distances for geographic data unless the boxcar step needs the reference formula
    const bool vec = GEO && P.e && F.e && kernel != GW_KERNEL_BOXCAR;

    double rmax = bw;
    if (t < CT_BM) {
        int i = row0 + t;
        bool ok = i < nf;
        sfu[t] = ok ? F.u[i] : 0.0;
        sfv[t] = ok ? F.v[i] : 0.0;
        sfuR[t] = (GEO && ok) ? F.uR[i] : 0.0;
        sfvR[t] = (GEO && ok) ? F.vR[i] : 0.0;
        const double r = ok ? (thr ? thr[i] : bw) : 0.0;
        sthr[t] = r;
        sr2[t] = r * r;
        sir2[t] = 1.0 / (r * r);
        for (int c = 0; c < 3; c++) sfe[c][t] = (vec && ok) ? F.e[(size_t)c * nf + i] : 0.0;
    }
    if (thr) {
        double r = (t < CT_BM && row0 + t < nf) ? thr[row0 + t] : -1.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, off));
        if ((t & 31) == 0) sred[t >> 5] = r;
    }
    if (t == 0) sbound = tb_union<GEO>(ftb16, row0 / CT_BK, (min(row0 + CT_BM, nf) - 1) / CT_BK);
    __syncthreads();
    if (thr) {
        rmax = sred[0];
        for (int q = 1; q < CT_THREADS / 32; q++) rmax = fmax(rmax, sred[q]);
    }
    // a tile may be skipped only if every pair in it has d >= r_i, i.e. w = 0
    const float4 fbound = sbound;
    const float far_thr = (skip_tiles && kernel >= GW_KERNEL_BISQUARE) ? tb_far_threshold<GEO>(rmax) : -1.0f;

    double acc[CT_ROWS_PER_THREAD][NC];
#pragma unroll
    for (int q = 0; q < CT_ROWS_PER_THREAD; q++)
#pragma unroll
        for (int c = 0; c < NC; c++) acc[q][c] = 0.0;

    const int ntiles = (n + CT_BK - 1) / CT_BK;
    for (int tile = 0; tile < ntiles; tile++) {
        if (tb_far<GEO>(fbound, tb16[tile], far_thr)) continue;  // uniform over the CTA
        const int j0 = tile * CT_BK;
        // Z tile -> shared (zero padded)
        for (int e = t; e < CT_BK * NCOL; e += CT_THREADS) {
            int k = e / NCOL, c = e - k * NCOL;
            int j = j0 + k;
            sZ[k][c] = (j < n && c < mcols) ? Z[(size_t)j * ldz + c] : 0.0;
        }
        // weight tile: thread (tx, ty) owns data point j0 + tx for rows ty + 16q
        {
            const int j = j0 + tx;
            double du = 0.0, dv = 0.0, duR = 0.0, dvR = 0.0, ex = 0.0, ey = 0.0, ez = 0.0;
            if (j < n) {
                du = P.u[j];
                dv = P.v[j];
                if (GEO) { duR = P.uR[j]; dvR = P.vR[j]; }
                if (vec) { ex = P.e[j]; ey = P.e[(size_t)n + j]; ez = P.e[2 * (size_t)n + j]; }
            }
#pragma unroll
            for (int q = 0; q < CT_ROWS_PER_THREAD; q++) {
                const int r = ty + 16 * q;
                const int i = row0 + r;
                double w = 0.0;
                if (j < n && i < nf) {
                    w = vec ? pair_weight64_vec(kernel, sfe[0][r], sfe[1][r], sfe[2][r], ex, ey, ez, sthr[r], sir2[r])
                            : pair_weight64<GEO>(kernel, du, dv, duR, dvR, sfu[r], sfv[r], sfuR[r], sfvR[r], sthr[r],
                                                 sr2[r], sir2[r]);
                    if (exclude_self && i == j) w = 0.0;
                    if (wpow == 2) w = w * w;
                }
                sW[r][tx] = w;
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < CT_BK; k++) {
            double a[CT_ROWS_PER_THREAD], b[NC];
#pragma unroll
            for (int q = 0; q < CT_ROWS_PER_THREAD; q++) a[q] = sW[ty + 16 * q][k];
#pragma unroll
            for (int c = 0; c < NC; c++) b[c] = sZ[k][tx + 16 * c];
#pragma unroll
            for (int q = 0; q < CT_ROWS_PER_THREAD; q++)
#pragma unroll
                for (int c = 0; c < NC; c++) acc[q][c] = fma(a[q], b[c], acc[q][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < CT_ROWS_PER_THREAD; q++) {
        const int i = row0 + ty + 16 * q;
        if (i >= nf) continue;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int col = tx + 16 * c;
            if (col < mcols) G[(size_t)i * ldg + col] = acc[q][c];
        }
    }
}

// Narrow form for mcols <= 4 (the one-variable problems of GWRMultiscale:
// m = 2 for the criterion, 1 for X^T W^2 X).  Thread (tx, ty) owns data point
// j0 + tx of each tile and rows ty + 16 q, keeps its weights in registers and
// accumulates M columns directly; the 16 partial sums of a row are reduced
// across the half-warp at the end.  No shared staging, no barrier per tile.
template <bool GEO, int M, int RPT>
__global__ void __launch_bounds__(CT_THREADS)
    k_contract64_narrow(DevPoints P, const float4* __restrict__ tb16, DevPoints F, const float4* __restrict__ ftb16,
                        const double* __restrict__ Z, int ldz, double* __restrict__ G, int ldg,
                        const double* __restrict__ thr, double bw, int kernel, int exclude_self, int wpow,
                        int skip_tiles)
{
    constexpr int BM = 16 * RPT;  // rows of this CTA
    __shared__ double sfu[BM], sfv[BM], sfuR[BM], sfvR[BM], sthr[BM], sr2[BM], sir2[BM];
    __shared__ double sfe[3][BM];
    __shared__ double sred[CT_THREADS / 32];
    __shared__ float4 sbound;

    const int n = P.n, nf = F.n;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int row0 = blockIdx.x * BM;
    const bool vec = GEO && P.e && F.e && kernel != GW_KERNEL_BOXCAR;

    double rmax = bw;
    if (t < BM) {
        int i = row0 + t;
        bool ok = i < nf;
        sfu[t] = ok ? F.u[i] : 0.0;
        sfv[t] = ok ? F.v[i] : 0.0;
        sfuR[t] = (GEO && ok) ? F.uR[i] : 0.0;
        sfvR[t] = (GEO && ok) ? F.vR[i] : 0.0;
        const double r = ok ? (thr ? thr[i] : bw) : 0.0;
        sthr[t] = r;
        sr2[t] = r * r;
        sir2[t] = 1.0 / (r * r);
        for (int c = 0; c < 3; c++) sfe[c][t] = (vec && ok) ? F.e[(size_t)c * nf + i] : 0.0;
    }
    if (thr) {
        double r = (t < BM && row0 + t < nf) ? thr[row0 + t] : -1.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, off));
        if ((t & 31) == 0) sred[t >> 5] = r;
    }
    if (t == 0) sbound = tb_union<GEO>(ftb16, row0 / CT_BK, (min(row0 + BM, nf) - 1) / CT_BK);
    __syncthreads();
    if (thr) {
        rmax = sred[0];
        for (int q = 1; q < CT_THREADS / 32; q++) rmax = fmax(rmax, sred[q]);
    }
    const float4 fbound = sbound;
    const float far_thr = (skip_tiles && kernel >= GW_KERNEL_BISQUARE) ? tb_far_threshold<GEO>(rmax) : -1.0f;

    double fu[RPT], fv[RPT], fuR[RPT], fvR[RPT], fex[RPT], fey[RPT], fez[RPT];
    double rr[RPT], rr2[RPT], rir2[RPT];
    int ri[RPT];
#pragma unroll
    for (int q = 0; q < RPT; q++) {
        const int r = ty + 16 * q;
        fu[q] = sfu[r];
        fv[q] = sfv[r];
        fuR[q] = sfuR[r];
        fvR[q] = sfvR[r];
        fex[q] = sfe[0][r];
        fey[q] = sfe[1][r];
        fez[q] = sfe[2][r];
        rr[q] = sthr[r];
        rr2[q] = sr2[r];
        rir2[q] = sir2[r];
        ri[q] = row0 + r < nf ? row0 + r : -1;
    }
    double acc[RPT][M];
#pragma unroll
    for (int q = 0; q < RPT; q++)
#pragma unroll
        for (int c = 0; c < M; c++) acc[q][c] = 0.0;

    const int ntiles = (n + CT_BK - 1) / CT_BK;
    for (int tile = 0; tile < ntiles; tile++) {
        if (tb_far<GEO>(fbound, tb16[tile], far_thr)) continue;  // uniform over the CTA
        const int j = tile * CT_BK + tx;
        if (j >= n) continue;
        const double du = P.u[j], dv = P.v[j];
        const double duR = GEO ? P.uR[j] : 0.0, dvR = GEO ? P.vR[j] : 0.0;
        const double ex = vec ? P.e[j] : 0.0, ey = vec ? P.e[(size_t)n + j] : 0.0,
                     ez = vec ? P.e[2 * (size_t)n + j] : 0.0;
        double z[M];
#pragma unroll
        for (int c = 0; c < M; c++) z[c] = Z[(size_t)j * ldz + c];
#pragma unroll
        for (int q = 0; q < RPT; q++) {
            if (ri[q] < 0) continue;
            double w = vec ? pair_weight64_vec(kernel, fex[q], fey[q], fez[q], ex, ey, ez, rr[q], rir2[q])
                           : pair_weight64<GEO>(kernel, du, dv, duR, dvR, fu[q], fv[q], fuR[q], fvR[q], rr[q],
                                                rr2[q], rir2[q]);
            if (exclude_self && ri[q] == j) w = 0.0;
            if (wpow == 2) w = w * w;
#pragma unroll
            for (int c = 0; c < M; c++) acc[q][c] = fma(w, z[c], acc[q][c]);
        }
    }
#pragma unroll
    for (int q = 0; q < RPT; q++)
#pragma unroll
        for (int c = 0; c < M; c++) {
            double v = acc[q][c];
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (tx == 0 && ri[q] >= 0) G[(size_t)ri[q] * ldg + c] = v;
        }
}

template <bool GEO, int NC>
cudaError_t launch_nc(const DevPoints& P, const float4* tiles, const DevPoints& F, const float4* ftiles,
                      const double* Z, int ldz, int mcols, double* G, int ldg, const double* thr, double bw,
                      int kernel, bool exclude_self, int wpow, bool skip, cudaStream_t s)
{
    int grid = (F.n + CT_BM - 1) / CT_BM;
    k_contract64<GEO, NC><<<grid, CT_THREADS, 0, s>>>(P, tiles, F, ftiles, Z, ldz, mcols, G, ldg, thr, bw, kernel,
                                                     exclude_self ? 1 : 0, wpow, skip ? 1 : 0);
    return cudaGetLastError();
}

template <bool GEO>
cudaError_t launch_geo(const DevPoints& P, const float4* tiles, const DevPoints& F, const float4* ftiles,
                       const double* Z, int ldz, int mcols, double* G, int ldg, const double* thr, double bw,
                       int kernel, bool exclude_self, int wpow, bool skip, cudaStream_t s)
{
    if (mcols <= 4) {
        // rows per CTA: 64 when that already gives a few CTAs per SM, else 32 or 16
        const int rpt = F.n >= 64 * 152 * 4 ? 4 : (F.n >= 32 * 152 * 4 ? 2 : 1);
        const int grid = (F.n + 16 * rpt - 1) / (16 * rpt);
        const int ex = exclude_self ? 1 : 0, sk = skip ? 1 : 0;
#define GW_NARROW(MM, R)                                                                                        \
    k_contract64_narrow<GEO, MM, R><<<grid, CT_THREADS, 0, s>>>(P, tiles, F, ftiles, Z, ldz, G, ldg, thr, bw, \
                                                                kernel, ex, wpow, sk)
#define GW_NARROW_M(MM)            \
    if (rpt == 4)                  \
        GW_NARROW(MM, 4);          \
    else if (rpt == 2)             \
        GW_NARROW(MM, 2);          \
    else                           \
        GW_NARROW(MM, 1);
        switch (mcols) {
        case 1: GW_NARROW_M(1) break;
        case 2: GW_NARROW_M(2) break;
        case 3: GW_NARROW_M(3) break;
        default: GW_NARROW_M(4) break;
        }
#undef GW_NARROW_M
#undef GW_NARROW
        return cudaGetLastError();
    }
    int nc = (mcols + 15) / 16;
#define GW_NC_CASE(K) \
    case K:           \
        return launch_nc<GEO, K>(P, tiles, F, ftiles, Z, ldz, mcols, G, ldg, thr, bw, kernel, exclude_self, wpow, \
                                 skip, s);
    switch (nc) {
        GW_NC_CASE(1) GW_NC_CASE(2) GW_NC_CASE(3) GW_NC_CASE(4) GW_NC_CASE(5) GW_NC_CASE(6) GW_NC_CASE(7)
        GW_NC_CASE(8) GW_NC_CASE(9) GW_NC_CASE(10) GW_NC_CASE(11) GW_NC_CASE(12) GW_NC_CASE(13)
        GW_NC_CASE(14) GW_NC_CASE(15) GW_NC_CASE(16)
    default: return cudaErrorInvalidValue;
    }
#undef GW_NC_CASE
}

}  // namespace

cudaError_t launch_contract64(const DevPoints& P, bool geographic, const float4* tb16, const double* Z, int ldz,
                              int mcols, double* G, int ldg, const double* thr, double bw, int kernel,
                              bool exclude_self, int wpow, bool skip_tiles, cudaStream_t stream)
{
    return launch_contract64_focus(P, tb16, P, tb16, geographic, Z, ldz, mcols, G, ldg, thr, bw, kernel, exclude_self,
                                   wpow, skip_tiles, stream);
}

cudaError_t launch_contract64_focus(const DevPoints& P, const float4* tb16, const DevPoints& F, const float4* ftb16,
                                    bool geographic, const double* Z, int ldz, int mcols, double* G, int ldg,
                                    const double* thr, double bw, int kernel, bool exclude_self, int wpow,
                                    bool skip_tiles, cudaStream_t stream)
{
    if (mcols < 1 || mcols > 256 || F.n < 1) return cudaErrorInvalidValue;
    if (geographic)
        return launch_geo<true>(P, tb16, F, ftb16, Z, ldz, mcols, G, ldg, thr, bw, kernel, exclude_self, wpow,
                                skip_tiles, stream);
    return launch_geo<false>(P, tb16, F, ftb16, Z, ldz, mcols, G, ldg, thr, bw, kernel, exclude_self, wpow,
                             skip_tiles, stream);
}

}  // namespace gwgpu
