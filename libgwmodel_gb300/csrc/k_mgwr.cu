// k_mgwr.cu -- device side of the GWRMultiscale hat matrix
// (GWRMultiscale.cpp:208-300 and :174-180).
//
// Every n x n matrix is row-major in the engine's sorted (Hilbert) order for
// both rows and columns.  The diagnostics only need tr(S0) and tr(S0^T S0),
// which are invariant under that symmetric permutation, so nothing is ever
// permuted back.
//
//  * k_mgwr_hat_all  the initial fit's projections (:216-224):
//                    SA_k(i, j) = w_ij x_ik (A_i^-1 x_j)_k and S0 = sum_k SA_k,
//                    from the local inverses the fit's solve stored.
//  * k_mgwr_sub      T = SA_k - S0          (the SArrayi of :298)
//  * k_mgwr_post     SA_k += S; S0 = SA_k - T (:299-300, after SA_k = S T)
//  * k_mgwr_traces   per-block partial sums of S0_ii and S0_ij^2.
#include "gw_kernels.h"

namespace gwgpu {

namespace {

constexpr int HA_THREADS = 128;
constexpr int HA_ROWS = 8;  // rows of A^-1 staged per pass

template <bool GEO>
__global__ void __launch_bounds__(HA_THREADS)
    k_mgwr_hat_all(DevPoints P, const double* __restrict__ X, int p, const double* __restrict__ ainv,
                   const double* __restrict__ thr, double bw, int kernel, double* __restrict__ S0,
                   double* __restrict__ SA)
{
    extern __shared__ double hsm[];
    double* sM = hsm;                    // HA_ROWS x p x p: x_ik A_i^-1(k, l)
    double* sX = sM + HA_ROWS * p * p;   // HA_THREADS x p: x_j of this block
    __shared__ double su[HA_ROWS], sv[HA_ROWS], suR[HA_ROWS], svR[HA_ROWS], sr[HA_ROWS];
    const int n = P.n, t = threadIdx.x;
    const int j0 = blockIdx.x * HA_THREADS, j = j0 + t;
    const size_t nn = (size_t)n * n;
    for (int e = t; e < HA_THREADS * p; e += HA_THREADS) {
        int jj = j0 + e / p;
        sX[e] = jj < n ? X[(size_t)j0 * p + e] : 0.0;
    }
    double du = 0.0, dv = 0.0, duR = 0.0, dvR = 0.0;
    if (j < n) {
        du = P.u[j];
        dv = P.v[j];
        if (GEO) {
            duR = P.uR[j];
            dvR = P.vR[j];
        }
    }
    for (int i0 = blockIdx.y * HA_ROWS; i0 < n; i0 += gridDim.y * HA_ROWS) {
        __syncthreads();
        if (t < HA_ROWS) {
            const int i = i0 + t;
            const bool ok = i < n;
            su[t] = ok ? P.u[i] : 0.0;
            sv[t] = ok ? P.v[i] : 0.0;
            suR[t] = (GEO && ok) ? P.uR[i] : 0.0;
            svR[t] = (GEO && ok) ? P.vR[i] : 0.0;
            sr[t] = ok ? (thr ? thr[i] : bw) : 0.0;
        }
        for (int e = t; e < HA_ROWS * p * p; e += HA_THREADS) {
            const int q = e / (p * p), k = (e / p) % p;
            const int i = i0 + q;
            sM[e] = i < n ? X[(size_t)i * p + k] * ainv[(size_t)i0 * p * p + e] : 0.0;
        }
        __syncthreads();
        if (j >= n) continue;
        const int iend = min(HA_ROWS, n - i0);
        for (int q = 0; q < iend; q++) {
            double d;
            if constexpr (GEO)
                d = kernel == GW_KERNEL_BOXCAR ? gw_gc_dist(du, su[q], dv, sv[q], duR, suR[q], dvR, svR[q])
                                               : gw_gc_dist_fast(du, su[q], dv, sv[q], duR, suR[q], dvR, svR[q]);
            else
                d = gw_planar_dist(du, dv, su[q], sv[q]);
            const double w = gw_kernel_weight(kernel, d, sr[q]);
            const size_t at = (size_t)(i0 + q) * n + j;
            double s0 = 0.0;
            for (int k = 0; k < p; k++) {
                double c = 0.0;
                for (int l = 0; l < p; l++) c += sM[(q * p + k) * p + l] * sX[t * p + l];
                const double s = w * c;
                SA[(size_t)k * nn + at] = s;
                s0 += s;
            }
            S0[at] = s0;
        }
    }
}

// SA(i, c0 + c) = v_i sum_j w_ij x_j (T(j, c0 + c) + [j == c0 + c]) for the 64
// rows of this CTA and HU_COLS columns from c0: the variable's hat matrix
// S(i, j) = w_ij v_i x_j (v_i = x_i / sum_j w_ij x_j^2) applied to T + I, over
// the data tiles that can hold a neighbour of a row of the CTA (compact
// kernels; gaussian and exponential weights visit every tile: the dense
// product).  The weight tile is computed in shared memory, the T tile is
// staged with the identity and the x_j scale folded in, and each thread
// accumulates 4 rows x HU_NC columns in FP64.
constexpr int HU_THREADS = 256;
constexpr int HU_BM = kRowBlock;  // 64 rows
constexpr int HU_BK = kTile;      // 16 data points
constexpr int HU_NC = 8;
constexpr int HU_COLS = 16 * HU_NC;  // 128 columns per CTA

template <bool GEO>
__global__ void __launch_bounds__(HU_THREADS)
    k_mgwr_hat_update(DevPoints P, const float4* __restrict__ tb16, const double* __restrict__ X,
                      const double* __restrict__ v, const double* __restrict__ thr, double bw, int kernel,
                      const double* __restrict__ T, double* __restrict__ SA)
{
    __shared__ double sW[HU_BM][HU_BK + 1];
    __shared__ double sT[HU_BK][HU_COLS];
    __shared__ double sfu[HU_BM], sfv[HU_BM], sfuR[HU_BM], sfvR[HU_BM], sthr[HU_BM];
    __shared__ double sred[HU_THREADS / 32];
    __shared__ float4 sbound;
    const int n = P.n;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int row0 = blockIdx.x * HU_BM;
    const int c0 = blockIdx.y * HU_COLS;
    if (t < HU_BM) {
        const int i = row0 + t;
        const bool ok = i < n;
        sfu[t] = ok ? P.u[i] : 0.0;
        sfv[t] = ok ? P.v[i] : 0.0;
        sfuR[t] = (GEO && ok) ? P.uR[i] : 0.0;
        sfvR[t] = (GEO && ok) ? P.vR[i] : 0.0;
        sthr[t] = ok ? (thr ? thr[i] : bw) : 0.0;
    }
    double rmax = bw;
    if (thr) {
        double r = (t < HU_BM && row0 + t < n) ? thr[row0 + t] : -1.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, off));
        if ((t & 31) == 0) sred[t >> 5] = r;
    }
    if (t == 0) sbound = tb_union<GEO>(tb16, row0 / HU_BK, (min(row0 + HU_BM, n) - 1) / HU_BK);
    __syncthreads();
    if (thr) {
        rmax = sred[0];
        for (int q = 1; q < HU_THREADS / 32; q++) rmax = fmax(rmax, sred[q]);
    }
    const float4 fbound = sbound;
    // compact kernels skip the tiles beyond every row's bandwidth; gaussian and exponential weights never vanish
    const float far_thr = kernel >= GW_KERNEL_BISQUARE ? tb_far_threshold<GEO>(rmax) : -1.0f;

    double acc[4][HU_NC];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
        for (int c = 0; c < HU_NC; c++) acc[q][c] = 0.0;

    const int ntiles = (n + HU_BK - 1) / HU_BK;
    for (int tile = 0; tile < ntiles; tile++) {
        if (tb_far<GEO>(fbound, tb16[tile], far_thr)) continue;  // uniform over the CTA
        const int j0 = tile * HU_BK;
        for (int e = t; e < HU_BK * HU_COLS; e += HU_THREADS) {
            const int k = e / HU_COLS, c = e - k * HU_COLS;
            const int j = j0 + k, col = c0 + c;
            double val = 0.0;
            if (j < n && col < n) val = X[j] * (T[(size_t)j * n + col] + (j == col ? 1.0 : 0.0));
            sT[k][c] = val;
        }
        {
            const int j = j0 + tx;
            double du = 0.0, dv = 0.0, duR = 0.0, dvR = 0.0;
            if (j < n) {
                du = P.u[j];
                dv = P.v[j];
                if (GEO) {
                    duR = P.uR[j];
                    dvR = P.vR[j];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int r = ty + 16 * q;
                double w = 0.0;
                if (j < n && row0 + r < n) {
                    double d;
                    if constexpr (GEO)
                        d = kernel == GW_KERNEL_BOXCAR ? gw_gc_dist(du, sfu[r], dv, sfv[r], duR, sfuR[r], dvR, sfvR[r])
                                                       : gw_gc_dist_fast(du, sfu[r], dv, sfv[r], duR, sfuR[r], dvR, sfvR[r]);
                    else
                        d = gw_planar_dist(du, dv, sfu[r], sfv[r]);
                    w = gw_kernel_weight(kernel, d, sthr[r]);
                }
                sW[r][tx] = w;
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < HU_BK; k++) {
            double a[4], b[HU_NC];
#pragma unroll
            for (int q = 0; q < 4; q++) a[q] = sW[ty + 16 * q][k];
#pragma unroll
            for (int c = 0; c < HU_NC; c++) b[c] = sT[k][tx + 16 * c];
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int c = 0; c < HU_NC; c++) acc[q][c] = fma(a[q], b[c], acc[q][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int i = row0 + ty + 16 * q;
        if (i >= n) continue;
        const double vi = v[i];
#pragma unroll
        for (int c = 0; c < HU_NC; c++) {
            const int col = c0 + tx + 16 * c;
            if (col < n) SA[(size_t)i * n + col] = vi * acc[q][c];
        }
    }
}

__global__ void k_mgwr_sub(size_t count, const double* __restrict__ SA, const double* __restrict__ S0,
                           double* __restrict__ T)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        T[e] = SA[e] - S0[e];
}

__global__ void k_mgwr_post(size_t count, double* __restrict__ SA, const double* __restrict__ S,
                            const double* __restrict__ T, double* __restrict__ S0)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const double a = S ? SA[e] + S[e] : SA[e];
        if (S) SA[e] = a;
        S0[e] = a - T[e];
    }
}

constexpr int TR_THREADS = 256;

__global__ void __launch_bounds__(TR_THREADS)
    k_mgwr_traces(int n, const double* __restrict__ S0, double* __restrict__ partials)
{
    __shared__ double sh[2][TR_THREADS];
    const size_t nn = (size_t)n * n;
    double tr = 0.0, ss = 0.0;
    for (size_t e = blockIdx.x * (size_t)TR_THREADS + threadIdx.x; e < nn; e += (size_t)gridDim.x * TR_THREADS) {
        const double s = S0[e];
        ss += s * s;
    }
    for (int i = blockIdx.x * TR_THREADS + threadIdx.x; i < n; i += gridDim.x * TR_THREADS)
        tr += S0[(size_t)i * (n + 1)];
    sh[0][threadIdx.x] = tr;
    sh[1][threadIdx.x] = ss;
    __syncthreads();
    for (int stride = TR_THREADS / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + stride];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + stride];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[blockIdx.x * 4 + 0] = sh[0][0];
        partials[blockIdx.x * 4 + 1] = sh[1][0];
        partials[blockIdx.x * 4 + 2] = 0.0;
        partials[blockIdx.x * 4 + 3] = 0.0;
    }
}

int elementwise_grid(size_t count)
{
    const size_t blocks = (count + 255) / 256;
    return (int)std::min<size_t>(blocks, 152 * 16);
}

}  // namespace

size_t mgwr_hat_all_smem(int p)
{
    return (size_t)(HA_ROWS * p * p + HA_THREADS * p) * sizeof(double);
}

cudaError_t launch_mgwr_hat_all(const DevPoints& P, bool geographic, const double* X, int p, const double* ainv,
                                const double* thr, double bw, int kernel, double* S0, double* SA, int num_sms,
                                cudaStream_t stream)
{
    const int gx = (P.n + HA_THREADS - 1) / HA_THREADS;
    // enough row groups that the grid covers every SM a few times over
    const int want = std::max(1, (num_sms * 8 + gx - 1) / gx);
    const int gy = std::min(want, (P.n + HA_ROWS - 1) / HA_ROWS);
    const size_t smem = mgwr_hat_all_smem(p);
    dim3 grid(gx, gy);
    if (geographic) {
        raise_smem_limit((const void*)k_mgwr_hat_all<true>, smem);
        k_mgwr_hat_all<true><<<grid, HA_THREADS, smem, stream>>>(P, X, p, ainv, thr, bw, kernel, S0, SA);
    } else {
        raise_smem_limit((const void*)k_mgwr_hat_all<false>, smem);
        k_mgwr_hat_all<false><<<grid, HA_THREADS, smem, stream>>>(P, X, p, ainv, thr, bw, kernel, S0, SA);
    }
    return cudaGetLastError();
}

cudaError_t launch_mgwr_hat_update(const DevPoints& P, bool geographic, const float4* tb16, const double* X,
                                   const double* v, const double* thr, double bw, int kernel, const double* T,
                                   double* SA, cudaStream_t stream)
{
    dim3 grid((P.n + HU_BM - 1) / HU_BM, (P.n + HU_COLS - 1) / HU_COLS);
    if (geographic)
        k_mgwr_hat_update<true><<<grid, HU_THREADS, 0, stream>>>(P, tb16, X, v, thr, bw, kernel, T, SA);
    else
        k_mgwr_hat_update<false><<<grid, HU_THREADS, 0, stream>>>(P, tb16, X, v, thr, bw, kernel, T, SA);
    return cudaGetLastError();
}

cudaError_t launch_mgwr_sub(size_t count, const double* SA, const double* S0, double* T, cudaStream_t stream)
{
    k_mgwr_sub<<<elementwise_grid(count), 256, 0, stream>>>(count, SA, S0, T);
    return cudaGetLastError();
}

cudaError_t launch_mgwr_post(size_t count, double* SA, const double* S, const double* T, double* S0,
                             cudaStream_t stream)
{
    k_mgwr_post<<<elementwise_grid(count), 256, 0, stream>>>(count, SA, S, T, S0);
    return cudaGetLastError();
}

cudaError_t launch_mgwr_traces(int n, const double* S0, double* partials, int max_blocks, int* nblocks,
                               cudaStream_t stream)
{
    const size_t nn = (size_t)n * n;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((nn + TR_THREADS - 1) / TR_THREADS, max_blocks));
    k_mgwr_traces<<<blocks, TR_THREADS, 0, stream>>>(n, S0, partials);
    *nblocks = blocks;
    return cudaGetLastError();
}

}  // namespace gwgpu
