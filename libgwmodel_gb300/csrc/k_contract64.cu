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

template <bool GEO, int NC>
__global__ void __launch_bounds__(CT_THREADS)
    k_contract64(DevPoints P, const float4* __restrict__ tb16, DevPoints F, const float4* __restrict__ ftb16,
                 const double* __restrict__ Z, int ldz, int mcols, double* __restrict__ G, int ldg,
                 const double* __restrict__ thr, double bw, int kernel, int exclude_self, int wpow, int skip_tiles)
{
    constexpr int NCOL = NC * 16;
    __shared__ double sW[CT_BM][CT_BK + 1];
    __shared__ double sZ[CT_BK][NCOL];
    __shared__ double sfu[CT_BM], sfv[CT_BM], sfuR[CT_BM], sfvR[CT_BM], sthr[CT_BM];
    __shared__ double sred[CT_THREADS / 32];
    __shared__ float4 sbound;

    const int n = P.n, nf = F.n;  // data points, focus rows (the data themselves, or prediction points)
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int row0 = blockIdx.x * CT_BM;

    double rmax = bw;
    if (t < CT_BM) {
        int i = row0 + t;
        bool ok = i < nf;
        sfu[t] = ok ? F.u[i] : 0.0;
        sfv[t] = ok ? F.v[i] : 0.0;
        sfuR[t] = (GEO && ok) ? F.uR[i] : 0.0;
        sfvR[t] = (GEO && ok) ? F.vR[i] : 0.0;
        sthr[t] = ok ? (thr ? thr[i] : bw) : 0.0;
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
            double du = 0.0, dv = 0.0, duR = 0.0, dvR = 0.0;
            if (j < n) {
                du = P.u[j];
                dv = P.v[j];
                if (GEO) { duR = P.uR[j]; dvR = P.vR[j]; }
            }
#pragma unroll
            for (int q = 0; q < CT_ROWS_PER_THREAD; q++) {
                const int r = ty + 16 * q;
                const int i = row0 + r;
                double w = 0.0;
                if (j < n && i < nf) {
                    double d;
                    if constexpr (GEO)
                        d = gw_gc_dist(du, sfu[r], dv, sfv[r], duR, sfuR[r], dvR, sfvR[r]);
                    else
                        d = gw_planar_dist(du, dv, sfu[r], sfv[r]);
                    w = gw_kernel_weight(kernel, d, sthr[r]);
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
