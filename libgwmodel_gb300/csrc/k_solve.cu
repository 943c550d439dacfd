// k_solve.cu -- per-location solves and the passes around the contraction.
//
//  * k_build_z      Z[j, :] = packed x_j x_j^T, x_j y_j (the contraction's B operand)
//  * k_solve        one warp per location: Cholesky of A_i = X^T W_i X (in
//                   place of inv_sympd, GWRBasic.cpp:507), beta_i, s_ii = w_ii
//                   x_i^T A_i^-1 x_i, the residual, and for the final fit
//                   v_i = A_i^-1 x_i, diag(A^-1 Q A^-1) (betasSE) and
//                   ||s_i||^2 = v_i^T Q_i v_i with Q_i = X^T W_i^2 X
//                   (GWRBasic.cpp:409-415); block partial sums of the criterion
//  * k_reduce       fixed-order sum of the block partials
//  * k_hat          qDiag_j = sum_i (delta_ij - s_ij)^2 and the rows of S
//                   (GWRBasic.cpp:416-419) without materialising C_i
//  * k_maxdist      CRSDistance::maxDistance (CRSDistance.cpp:133-143)
#include "gw_common.cuh"
#include "gw_kernels.h"
#include "mixed_weight.cuh"

namespace gwgpu {

namespace {

constexpr int SV_WARPS = 4;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int packed_index(int a, int b, int p)
{
    // a <= b, upper triangle packed by rows
    return a * p - (a * (a - 1)) / 2 + (b - a);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
    return v;
}

__global__ void k_build_z(int n, int p, const double* __restrict__ X, const double* __restrict__ y,
                          double* __restrict__ Z)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int mm = p * (p + 1) / 2, m = mm + p;
    const double* x = X + (size_t)j * p;
    double* z = Z + (size_t)j * m;
    int e = 0;
    for (int a = 0; a < p; a++)
        for (int b = a; b < p; b++) z[e++] = x[a] * x[b];
    for (int a = 0; a < p; a++) z[mm + a] = x[a] * y[j];
}

// The factor keeps 1 / L_jj on its diagonal, so the substitutions multiply.
// Forward substitution L z = rhs (lane r holds rhs_r; returns z_r).
__device__ __forceinline__ double fwd_solve(const double* L, int ld, int p, int lane, double rhs)
{
    double v = rhs;
    for (int j = 0; j < p; j++) {
        double zj = __shfl_sync(FULL, v, j) * L[j * ld + j];
        if (lane == j) v = zj;
        else if (lane > j && lane < p) v -= L[lane * ld + j] * zj;
    }
    return v;
}

// Two forward substitutions with the same factor in one pass (the same
// arithmetic as two fwd_solve calls, interleaved for latency).
__device__ __forceinline__ void fwd_solve2(const double* L, int ld, int p, int lane, double& v1, double& v2)
{
    for (int j = 0; j < p; j++) {
        const double ljj = L[j * ld + j];
        const double z1 = __shfl_sync(FULL, v1, j) * ljj;
        const double z2 = __shfl_sync(FULL, v2, j) * ljj;
        if (lane == j) {
            v1 = z1;
            v2 = z2;
        } else if (lane > j && lane < p) {
            const double l = L[lane * ld + j];
            v1 -= l * z1;
            v2 -= l * z2;
        }
    }
}

// Backward substitution L^T x = rhs.
__device__ __forceinline__ double bwd_solve(const double* L, int ld, int p, int lane, double rhs)
{
    double v = rhs;
    for (int j = p - 1; j >= 0; j--) {
        double xj = __shfl_sync(FULL, v, j) * L[j * ld + j];
        if (lane == j) v = xj;
        else if (lane < j) v -= L[j * ld + lane] * xj;
    }
    return v;
}

// BATCH: block b solves rows [work[b].y, work[b].z) of segment work[b].x
// (arguments segs[work[b].x]) and writes its partial sums to slot work[b].w
// of that segment's partials; otherwise the blocks stride over all rows.
template <int MODE, bool BATCH>
__global__ void __launch_bounds__(SV_WARPS * 32)
    k_solve(SolveArgs a0, const SolveArgs* __restrict__ segs, const int4* __restrict__ work)
{
    const int4 wk = BATCH ? work[blockIdx.x] : make_int4(0, 0, 0, 0);
    const SolveArgs a = BATCH ? segs[wk.x] : a0;
    extern __shared__ double smem[];
    const int p = a.p, ld = p + 1, mm = p * (p + 1) / 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per_warp = (MODE == kSolveFit) ? 4 * p * ld + 2 * p : p * ld + p;
    double* L = smem + warp * per_warp;
    double* Ainv = L + p * ld;
    double* Q = Ainv + p * ld;
    double* T = Q + p * ld;
    double* vsh = (MODE == kSolveFit) ? T + p * ld : L + p * ld;
    double* tsh = vsh + p;
    __shared__ double part[SV_WARPS][4];

    double acc_s = 0.0, acc_r = 0.0, acc_t = 0.0, acc_f = 0.0;
    const int row_first = BATCH ? wk.y + warp : blockIdx.x * SV_WARPS + warp;
    const int row_end = BATCH ? wk.z : a.n;
    const int row_step = BATCH ? SV_WARPS : gridDim.x * SV_WARPS;
    for (int row = row_first; row < row_end; row += row_step) {
        const double* g = a.G + (size_t)row * a.ldg;
        if (lane < p)
            for (int c = 0; c <= lane; c++) L[lane * ld + c] = g[packed_index(c, lane, p)];
        const double bvec = lane < p ? g[mm + lane] : 0.0;
        const double xr = (MODE != kSolvePredict && lane < p) ? a.X[(size_t)row * p + lane] : 0.0;
        __syncwarp();
        // Right-looking Cholesky: after column j is scaled, the trailing
        // triangle (j < c <= r < p) takes A_rc -= L_rj L_cj with its
        // (p-1-j)(p-j)/2 elements spread over all 32 lanes.  Every element sees
        // the same subtractions in the same order as a left-looking (Crout)
        // factorisation, so the factor is the same to the bit.
        bool fail = false;
        for (int j = 0; j < p; j++) {
            const double tjj = L[j * ld + j];
            if (!(tjj > 0.0)) { fail = true; break; }
            const double rinv = rsqrt(tjj);  // 1 / L_jj
            __syncwarp();
            if (lane == j) L[j * ld + j] = rinv;
            else if (lane > j && lane < p) L[lane * ld + j] *= rinv;
            __syncwarp();
            const int m = p - 1 - j, tri = m * (m + 1) / 2;
            for (int e = lane; e < tri; e += 32) {
                // e -> (rr, cc), cc <= rr: rr = floor((sqrt(8e + 1) - 1) / 2), exact for e < 528
                const int rr = (int)((sqrtf((float)(8 * e + 1)) - 1.0f) * 0.5f);
                const int cc = e - rr * (rr + 1) / 2;
                const int r = j + 1 + rr, c = j + 1 + cc;
                L[r * ld + c] -= L[r * ld + j] * L[c * ld + j];
            }
            __syncwarp();
        }
        if (fail) {
            if (a.beta && lane < p) a.beta[(size_t)row * p + lane] = __longlong_as_double(0x7ff8000000000000ll);
            if (lane == 0) {
                acc_f += 1.0;
                if (MODE != kSolvePredict) {
                    a.resid[row] = __longlong_as_double(0x7ff8000000000000ll);
                    a.sii[row] = 0.0;
                }
            }
            __syncwarp();
            continue;
        }
        if (MODE == kSolveAIC || MODE == kSolveCV) {
            // z = L^-1 b and u = L^-1 x_i: yhat_i = x_i^T A^-1 b = u . z and
            // x_i^T A^-1 x_i = u . u, so the criterion needs no backward
            // substitution; beta only when the caller asks for it
            double z = bvec, u = xr;
            fwd_solve2(L, ld, p, lane, z, u);
            const double yhat = warp_sum(lane < p ? u * z : 0.0);
            const double res = a.y[row] - yhat;
            double sii = 0.0;
            if (MODE == kSolveAIC) {
                const double uu = warp_sum(lane < p ? u * u : 0.0);
                sii = gw_kernel_weight(a.kernel, 0.0, a.thr ? a.thr[row] : a.bw) * uu;
            }
            if (a.beta) {
                const double beta = bwd_solve(L, ld, p, lane, z);
                if (lane < p) a.beta[(size_t)row * p + lane] = beta;
            }
            if (lane == 0) {
                a.sii[row] = sii;
                a.resid[row] = res;
                acc_s += sii;
                acc_r += res * res;
            }
            __syncwarp();
            continue;
        }
        double beta;
        if (MODE == kSolveRefine) {
            const double rv = lane < p ? a.rvec[(size_t)row * p + lane] : 0.0;
            const double delta = bwd_solve(L, ld, p, lane, fwd_solve(L, ld, p, lane, rv));
            beta = (lane < p ? a.beta[(size_t)row * p + lane] : 0.0) + delta;
        } else {
            beta = bwd_solve(L, ld, p, lane, fwd_solve(L, ld, p, lane, bvec));
        }
        if (lane < p) a.beta[(size_t)row * p + lane] = beta;
        if (MODE == kSolvePredict) {
            // a prediction point has no x_i or y_i: beta is the whole output (GWRBasic.cpp:166-190)
            __syncwarp();
            continue;
        }
        const double yhat = warp_sum(lane < p ? xr * beta : 0.0);
        const double res = a.y[row] - yhat;
        double sii = 0.0;
        if (MODE == kSolveRefine) {
            sii = a.sii[row];
        } else if (MODE != kSolveCV) {
            const double u = fwd_solve(L, ld, p, lane, xr);
            const double uu = warp_sum(lane < p ? u * u : 0.0);
            const double rr = a.thr ? a.thr[row] : a.bw;
            sii = gw_kernel_weight(a.kernel, 0.0, rr) * uu;
            if (MODE == kSolveFit) {
                const double v = bwd_solve(L, ld, p, lane, u);
                if (lane < p) {
                    a.v[(size_t)row * p + lane] = v;
                    vsh[lane] = v;
                }
                // U = L^-1 (lower triangular), lane j computing column j by forward
                // substitution (L keeps 1 / L_jj on its diagonal), into T
                if (lane < p) {
                    const int j = lane;
                    T[j * ld + j] = L[j * ld + j];
                    for (int r2 = j + 1; r2 < p; r2++) {
                        double acc = 0.0;
                        for (int k = j; k < r2; k++) acc = fma(L[r2 * ld + k], T[k * ld + j], acc);
                        T[r2 * ld + j] = -acc * L[r2 * ld + r2];
                    }
                }
                __syncwarp();
                // A^-1 = U^T U over the p (p + 1) / 2 elements (c, r), c <= r, spread over the
                // lanes: sum over k >= r of U_kc U_kr
                const int tri = p * (p + 1) / 2;
                for (int e = lane; e < tri; e += 32) {
                    const int rr = (int)((sqrtf((float)(8 * e + 1)) - 1.0f) * 0.5f);  // exact for e < 528
                    const int cc = e - rr * (rr + 1) / 2;
                    double acc = 0.0;
                    for (int k = rr; k < p; k++) acc = fma(T[k * ld + cc], T[k * ld + rr], acc);
                    Ainv[cc * ld + rr] = acc;
                    Ainv[rr * ld + cc] = acc;
                }
                __syncwarp();
                if (a.ainv && lane < p)
                    for (int k = 0; k < p; k++) a.ainv[((size_t)row * p + lane) * p + k] = Ainv[lane * ld + k];
                const double* g2 = a.G2 + (size_t)row * a.ldg2;
                if (lane < p)
                    for (int c = 0; c < p; c++)
                        Q[lane * ld + c] = g2[lane <= c ? packed_index(lane, c, p) : packed_index(c, lane, p)];
                if (lane < p) tsh[lane] = a.tvec ? a.tvec[lane] : 0.0;
                __syncwarp();
                // W = Q A^-1 (into T; U is done) over the p^2 elements, and (Q v)_lane
                for (int e = lane; e < p * p; e += 32) {
                    const int ra = e / p, cb = e - ra * p;
                    double acc = 0.0;
                    for (int q = 0; q < p; q++) acc = fma(Q[ra * ld + q], Ainv[q * ld + cb], acc);
                    T[ra * ld + cb] = acc;
                }
                double qv = 0.0;
                if (lane < p)
                    for (int b = 0; b < p; b++) qv = fma(Q[lane * ld + b], vsh[b], qv);
                __syncwarp();
                // diag(A^-1 Q A^-1)_k = sum_a A^-1_ka W_ak
                double mdiag = 0.0;
                if (lane < p)
                    for (int q = 0; q < p; q++) mdiag = fma(Ainv[lane * ld + q], T[q * ld + lane], mdiag);
                // t^T A^-1 Q A^-1 t = z^T Q z with z = A^-1 t (the intercept row after centring)
                double tmt = 0.0;
                if (a.tvec) {
                    double* zsh = L;  // the factor is no longer needed
                    double z = 0.0;
                    if (lane < p)
                        for (int q = 0; q < p; q++) z = fma(Ainv[lane * ld + q], tsh[q], z);
                    __syncwarp();
                    if (lane < p) zsh[lane] = z;
                    __syncwarp();
                    double qz = 0.0;
                    if (lane < p)
                        for (int b = 0; b < p; b++) qz = fma(Q[lane * ld + b], zsh[b], qz);
                    tmt = warp_sum(lane < p ? z * qz : 0.0);
                }
                const double ti = (a.tinv && lane < p) ? a.tinv[lane] : 1.0;
                if (lane < p) a.bse[(size_t)row * p + lane] = (a.tvec && lane == a.tcol) ? tmt : ti * ti * mdiag;
                const double sts = warp_sum(lane < p ? vsh[lane] * qv : 0.0);
                if (lane == 0) acc_t += sts;
            }
        }
        if (lane == 0) {
            a.sii[row] = sii;
            a.resid[row] = res;
            acc_s += sii;
            acc_r += res * res;
        }
        __syncwarp();
    }
    if (lane == 0) {
        part[warp][0] = acc_s;
        part[warp][1] = acc_r;
        part[warp][2] = acc_t;
        part[warp][3] = acc_f;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < SV_WARPS; w++) s += part[w][threadIdx.x];
        a.partials[(BATCH ? wk.w : blockIdx.x) * 4 + threadIdx.x] = s;
    }
}

constexpr int ST_THREADS = 32;  // locations (lanes) per block of k_solve_crit_t

// Criterion solves (AICc / CV, no beta) with one location per thread.  GB300
// runs FP64 at about two lanes per clock per SM, so an FP64 warp instruction
// costs the same whatever its active lanes: the warp-per-location form above
// spends most of its instructions on a few lanes (the tail of each trailing
// update, the pivots, the substitutions).  Here every lane has its own p x p
// factor in shared memory (element e of lane t at e * ST_THREADS + t, so a
// warp's accesses hit 32 consecutive doubles), and each operation is the one
// the warp form applies to that element, in the same order, down to the
// butterfly order of its warp sums (where the compiler fuses a product into a
// sum differently the two can differ by an ulp).  Only the grouping of the
// block partials of the criterion sums differs.
__device__ __forceinline__ int tri_index(int r, int c) { return r * (r + 1) / 2 + c; }  // c <= r

// Lane 0's value of warp_sum over x[i] y[i], i < p, padded with zeros to 32
// (x, y: one lane's column of a shared-memory block, stride ST_THREADS).
__device__ __forceinline__ double butterfly_dot(const double* x, const double* y, int p)
{
    double a[32];
#pragma unroll
    for (int i = 0; i < 32; i++) a[i] = i < p ? x[(size_t)i * ST_THREADS] * y[(size_t)i * ST_THREADS] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int i = 0; i < off; i++) a[i] = a[i] + a[i + off];
    }
    return a[0];
}

template <int MODE>
__global__ void __launch_bounds__(ST_THREADS) k_solve_crit_t(SolveArgs a)
{
    extern __shared__ double smem[];
    const int p = a.p, mm = p * (p + 1) / 2, m = mm + p;
    const int t = threadIdx.x;
    double* L = smem;                      // mm elements (lower, packed by rows) x ST_THREADS
    double* zv = smem + (size_t)mm * ST_THREADS;  // p elements
    double* uv = zv + (size_t)p * ST_THREADS;     // p elements
    // element of column q of G in the shared block: A[c][r] (upper, packed by
    // rows) goes to the lower factor's tri_index(r, c), b right after it; built
    // once, so the loads below need no division or search per element
    __shared__ short slot[20 * 21 / 2 + 20];
    for (int q = t; q < m; q += ST_THREADS) {
        if (q < mm) {
            int c = 0, base = 0;
            while (base + (p - c) <= q) {
                base += p - c;
                c++;
            }
            slot[q] = (short)tri_index(c + (q - base), c);
        } else {
            slot[q] = (short)q;  // zv follows L: element mm + (q - mm)
        }
    }
    double acc_s = 0.0, acc_r = 0.0, acc_f = 0.0;
    for (int row0 = blockIdx.x * ST_THREADS; row0 < a.n; row0 += gridDim.x * ST_THREADS) {
        const int nrow = min(ST_THREADS, a.n - row0);
        __syncwarp();
        // coalesced loads of the block's rows of G, four rows (up to 32 loads per lane) in
        // flight before their stores: G streams from DRAM, and one row at a time left
        // the loads waiting on each other
        for (int lr0 = 0; lr0 < nrow; lr0 += 4) {
            double v[4][8];  // m <= 230 columns: at most 8 per lane
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const double* g = a.G + (size_t)(row0 + lr0 + u) * a.ldg;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int q = t + k * ST_THREADS;
                    v[u][k] = (lr0 + u < nrow && q < m) ? g[q] : 0.0;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int q = t + k * ST_THREADS;
                    if (lr0 + u < nrow && q < m) L[(size_t)slot[q] * ST_THREADS + lr0 + u] = v[u][k];
                }
            }
        }
        __syncwarp();
        const int row = row0 + t;
        if (t < nrow) {
            double* Lt = L + t;
            double* zt = zv + t;
            double* ut = uv + t;
            for (int r = 0; r < p; r++) ut[(size_t)r * ST_THREADS] = a.X[(size_t)row * p + r];
            bool fail = false;
            for (int j = 0; j < p; j++) {
                const double tjj = Lt[(size_t)tri_index(j, j) * ST_THREADS];
                if (!(tjj > 0.0)) {
                    fail = true;
                    break;
                }
                const double rinv = rsqrt(tjj);
                Lt[(size_t)tri_index(j, j) * ST_THREADS] = rinv;
                for (int r = j + 1; r < p; r++) Lt[(size_t)tri_index(r, j) * ST_THREADS] *= rinv;
                for (int r = j + 1; r < p; r++) {
                    const double lrj = Lt[(size_t)tri_index(r, j) * ST_THREADS];
                    for (int c = j + 1; c <= r; c++) {
                        double* lrc = Lt + (size_t)tri_index(r, c) * ST_THREADS;
                        *lrc -= lrj * Lt[(size_t)tri_index(c, j) * ST_THREADS];
                    }
                }
            }
            if (fail) {
                acc_f += 1.0;
                if (a.beta) for (int r = 0; r < p; r++) a.beta[(size_t)row * p + r] = __longlong_as_double(0x7ff8000000000000ll);
                a.resid[row] = __longlong_as_double(0x7ff8000000000000ll);
                a.sii[row] = 0.0;
            } else {
                // z = L^-1 b and u = L^-1 x_i (fwd_solve2)
                for (int j = 0; j < p; j++) {
                    const double ljj = Lt[(size_t)tri_index(j, j) * ST_THREADS];
                    const double z1 = zt[(size_t)j * ST_THREADS] * ljj;
                    const double z2 = ut[(size_t)j * ST_THREADS] * ljj;
                    zt[(size_t)j * ST_THREADS] = z1;
                    ut[(size_t)j * ST_THREADS] = z2;
                    for (int r = j + 1; r < p; r++) {
                        const double l = Lt[(size_t)tri_index(r, j) * ST_THREADS];
                        zt[(size_t)r * ST_THREADS] -= l * z1;
                        ut[(size_t)r * ST_THREADS] -= l * z2;
                    }
                }
                const double yhat = butterfly_dot(ut, zt, p);
                const double res = a.y[row] - yhat;
                double sii = 0.0;
                if (MODE == kSolveAIC) {
                    const double uu = butterfly_dot(ut, ut, p);
                    sii = gw_kernel_weight(a.kernel, 0.0, a.thr ? a.thr[row] : a.bw) * uu;
                }
                a.sii[row] = sii;
                a.resid[row] = res;
                acc_s += sii;
                acc_r += res * res;
            }
        }
    }
    // the block's partial sums (lane order)
    __shared__ double part[ST_THREADS][3];
    part[t][0] = acc_s;
    part[t][1] = acc_r;
    part[t][2] = acc_f;
    __syncwarp();
    if (t < 4) {
        double v = 0.0;
        if (t != 2)
            for (int q = 0; q < ST_THREADS; q++) v += part[q][t == 3 ? 2 : t];
        a.partials[blockIdx.x * 4 + t] = v;
    }
}

__global__ void k_reduce(const double* __restrict__ partials, int nblocks, double* __restrict__ out)
{
    __shared__ double sh[256][4];
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += 256)
        for (int q = 0; q < 4; q++) s[q] += partials[b * 4 + q];
    for (int q = 0; q < 4; q++) sh[threadIdx.x][q] = s[q];
    __syncthreads();
    for (int stride = 128; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride)
            for (int q = 0; q < 4; q++) sh[threadIdx.x][q] += sh[threadIdx.x + stride][q];
        __syncthreads();
    }
    if (threadIdx.x < 4) out[threadIdx.x] = sh[0][threadIdx.x];
}

constexpr int HAT_THREADS = 128;
constexpr int HAT_TILE = kTile;

template <bool GEO>
__global__ void __launch_bounds__(HAT_THREADS)
    k_hat(DevPoints P, const float4* __restrict__ tb16, const float* __restrict__ tile_thr,
          const double* __restrict__ X, int p,
          const double* __restrict__ v, const double* __restrict__ thr, double bw, int kernel, int skip,
          double* __restrict__ qdiag, double* __restrict__ S, int row_target, double* __restrict__ s_row)
{
    extern __shared__ double hsm[];
    double* sX = hsm;                          // HAT_THREADS x p (x_j of this block)
    double* sV = sX + HAT_THREADS * p;         // HAT_TILE x p   (v_i of the staged rows)
    __shared__ double su[HAT_TILE], sv[HAT_TILE], suR[HAT_TILE], svR[HAT_TILE], sr[HAT_TILE];
    __shared__ float4 sbound;
    const int n = P.n, t = threadIdx.x;
    const int j0 = blockIdx.x * HAT_THREADS, j = j0 + t;
    for (int e = t; e < HAT_THREADS * p; e += HAT_THREADS) {
        int jj = j0 + e / p;
        sX[e] = jj < n ? X[(size_t)j0 * p + e] : 0.0;
    }
    if (t == 0) sbound = tb_union<GEO>(tb16, j0 / HAT_TILE, (min(j0 + HAT_THREADS, n) - 1) / HAT_TILE);
    __syncthreads();
    double du = 0.0, dv = 0.0, duR = 0.0, dvR = 0.0;
    if (j < n) {
        du = P.u[j]; dv = P.v[j];
        if (GEO) { duR = P.uR[j]; dvR = P.vR[j]; }
    }
    const bool can_skip = skip && tile_thr && kernel >= GW_KERNEL_BISQUARE;
    const float4 fbound = sbound;
    double acc = 0.0;
    const int ntiles = (n + HAT_TILE - 1) / HAT_TILE;
    for (int tile = 0; tile < ntiles; tile++) {
        const int i0 = tile * HAT_TILE;
        if (can_skip && tb_far<GEO>(fbound, tb16[tile], tile_thr[tile])) continue;  // uniform over the CTA
        if (t < HAT_TILE) {
            int i = i0 + t;
            bool ok = i < n;
            su[t] = ok ? P.u[i] : 0.0;
            sv[t] = ok ? P.v[i] : 0.0;
            suR[t] = (GEO && ok) ? P.uR[i] : 0.0;
            svR[t] = (GEO && ok) ? P.vR[i] : 0.0;
            sr[t] = ok ? (thr ? thr[i] : bw) : 0.0;
        }
        for (int e = t; e < HAT_TILE * p; e += HAT_THREADS) {
            int i = i0 + e / p;
            sV[e] = i < n ? v[(size_t)i0 * p + e] : 0.0;
        }
        __syncthreads();
        if (j < n) {
            const int iend = min(HAT_TILE, n - i0);
            for (int q = 0; q < iend; q++) {
                double d;
                if constexpr (GEO)
                    d = kernel == GW_KERNEL_BOXCAR ? gw_gc_dist(du, su[q], dv, sv[q], duR, suR[q], dvR, svR[q])
                                                   : gw_gc_dist_fast(du, su[q], dv, sv[q], duR, suR[q], dvR, svR[q]);
                else
                    d = gw_planar_dist(du, dv, su[q], sv[q]);
                double w = gw_kernel_weight(kernel, d, sr[q]);
                double dot = 0.0;
                for (int r = 0; r < p; r++) dot += sV[q * p + r] * sX[t * p + r];
                double s = w * dot;
                double e = (i0 + q == j) ? 1.0 - s : -s;
                acc += e * e;
                if (S) S[(size_t)(i0 + q) * n + j] = s;
                if (i0 + q == row_target) s_row[j] = s;
            }
        }
        __syncthreads();
    }
    if (j < n) qdiag[j] = acc;
}

// Mixed-precision hat pass: the weights are the FP32 weights of the tensor-core
// contraction (FP32 proxy distance, FP32 threshold); the hat entries
// s_ij = w_ij v_i^T x_j in FP32, the sums of squares in FP64.
template <bool GEO>
__global__ void __launch_bounds__(HAT_THREADS)
    k_hat_mixed(int n, const float4* __restrict__ pts, const float4* __restrict__ tb16,
                const float* __restrict__ tile_thr, const double* __restrict__ X, int p,
                const double* __restrict__ v, const float* __restrict__ thr32, float bw, int kernel,
                double* __restrict__ qdiag, double* __restrict__ S, int row_target, double* __restrict__ s_row)
{
    // FP32 copies of x_j and v_i: the FP32 weights already give s_ij a ~1e-7
    // relative error, and an FP32 dot product of p terms adds one of the same
    // order at 1/64 of the FP64 cost per pair; qDiag_j = sum_i (delta_ij - s_ij)^2
    // is dominated by (1 - s_jj)^2 with s_jj ~ p / b, so it moves by far less
    extern __shared__ float hsmf[];
    float* sX = hsmf;                      // HAT_THREADS x p
    float* sV = sX + HAT_THREADS * p;      // HAT_TILE x p
    constexpr int NF = GEO ? 2 : 1;
    __shared__ float4 sf[HAT_TILE][NF];
    __shared__ float sr[HAT_TILE], sinv[HAT_TILE];
    __shared__ float4 sbound;
    const int t = threadIdx.x;
    const int j0 = blockIdx.x * HAT_THREADS, j = j0 + t;
    for (int e = t; e < HAT_THREADS * p; e += HAT_THREADS) {
        int jj = j0 + e / p;
        sX[e] = jj < n ? (float)X[(size_t)j0 * p + e] : 0.0f;
    }
    if (t == 0) sbound = tb_union<GEO>(tb16, j0 / HAT_TILE, (min(j0 + HAT_THREADS, n) - 1) / HAT_TILE);
    __syncthreads();
    float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;
    if (j < n) {
        pa = pts[NF * (size_t)j];
        if (GEO) pb = pts[2 * (size_t)j + 1];
    }
    const bool can_skip = tile_thr && kernel >= GW_KERNEL_BISQUARE;
    const float4 fbound = sbound;
    double acc = 0.0;
    const int ntiles = (n + HAT_TILE - 1) / HAT_TILE;
    for (int tile = 0; tile < ntiles; tile++) {
        const int i0 = tile * HAT_TILE;
        if (can_skip && tb_far<GEO>(fbound, tb16[tile], tile_thr[tile])) continue;  // uniform over the CTA
        if (t < HAT_TILE) {
            const int i = i0 + t;
            const bool ok = i < n;
            for (int q = 0; q < NF; q++) sf[t][q] = ok ? pts[NF * (size_t)i + q] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float r = ok ? (thr32 ? thr32[i] : bw) : 1.0f;
            sr[t] = r;
            sinv[t] = 1.0f / (r * r);
        }
        for (int e = t; e < HAT_TILE * p; e += HAT_THREADS) {
            int i = i0 + e / p;
            sV[e] = i < n ? (float)v[(size_t)i0 * p + e] : 0.0f;
        }
        __syncthreads();
        if (j < n) {
            const int iend = min(HAT_TILE, n - i0);
            for (int q = 0; q < iend; q++) {
                const float d2 = GEO ? geo_d2_32(sf[q][0], sf[q][1], pa, pb) : planar_d2_32(sf[q][0], pa);
                const float w = weight32(kernel, d2, sr[q], sinv[q]);
                double s = 0.0;
                if (w != 0.0f) {
                    float dot = 0.0f;
                    for (int r = 0; r < p; r++) dot = fmaf(sV[q * p + r], sX[t * p + r], dot);
                    s = (double)(w * dot);
                }
                const double e = (i0 + q == j) ? 1.0 - s : -s;
                acc += e * e;
                if (S) S[(size_t)(i0 + q) * n + j] = s;
                if (i0 + q == row_target) s_row[j] = s;
            }
        }
        __syncthreads();
    }
    if (j < n) qdiag[j] = acc;
}

// CRSDistance::maxDistance (CRSDistance.cpp:133-143).  Planar distances are
// exact, so one pass takes the maximum.  Great-circle distances take two: the
// first finds every row's maximum with the unit-vector form of the formula
// (a few ulp, ~100 FP64 operations per pair instead of the ~3,000 of the
// correctly rounded one); the second evaluates the reference's double only
// for the pairs of the rows that come within kMaxdistMargin of the largest
// row maximum, so the result is the reference's maximum.
constexpr double kMaxdistMargin = 1e-9;

template <bool GEO>
__global__ void k_maxdist(DevPoints P, unsigned long long* __restrict__ key, double* __restrict__ rowmax)
{
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x / 32);
    double best = 0.0;
    for (int i = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); i < P.n; i += warps) {
        const double fu = P.u[i], fv = P.v[i];
        double rm = 0.0;
        if constexpr (GEO) {
            const double fuR = P.uR[i], fvR = P.vR[i];
            if (P.e) {
                const double xi = P.e[i], yi = P.e[(size_t)P.n + i], zi = P.e[2 * (size_t)P.n + i];
                for (int j = lane; j < P.n; j += 32)
                    rm = fmax(rm, gc_dist_vec(xi, yi, zi, P.e[j], P.e[(size_t)P.n + j], P.e[2 * (size_t)P.n + j]));
            } else {
                for (int j = lane; j < P.n; j += 32)
                    rm = fmax(rm, gw_gc_dist_fast(P.u[j], fu, P.v[j], fv, P.uR[j], fuR, P.vR[j], fvR));
            }
        } else {
            for (int j = lane; j < P.n; j += 32) rm = fmax(rm, gw_planar_dist(P.u[j], P.v[j], fu, fv));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) rm = fmax(rm, __shfl_xor_sync(FULL, rm, off));
        if (GEO && lane == 0) rowmax[i] = rm;
        best = fmax(best, rm);
    }
    if (lane == 0) atomicMax(key, (unsigned long long)dkey(best));
}

// Second pass of the great-circle maximum: key[0] holds the first pass's
// maximum M; rows whose maximum reaches M (1 - margin) evaluate the
// reference's double for their pairs within the margin into key[1].
__global__ void k_maxdist_exact(DevPoints P, unsigned long long* __restrict__ key, const double* __restrict__ rowmax)
{
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x / 32);
    const double cut = keyd(key[0]) * (1.0 - kMaxdistMargin);
    double best = 0.0;
    for (int i = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); i < P.n; i += warps) {
        if (!(rowmax[i] >= cut)) continue;  // warp-uniform
        const double fu = P.u[i], fv = P.v[i], fuR = P.uR[i], fvR = P.vR[i];
        for (int j = lane; j < P.n; j += 32) {
            const double df = P.e ? gc_dist_vec(P.e[i], P.e[(size_t)P.n + i], P.e[2 * (size_t)P.n + i], P.e[j],
                                                P.e[(size_t)P.n + j], P.e[2 * (size_t)P.n + j])
                                  : gw_gc_dist_fast(P.u[j], fu, P.v[j], fv, P.uR[j], fuR, P.vR[j], fvR);
            if (df >= cut) best = fmax(best, gw_gc_dist(P.u[j], fu, P.v[j], fv, P.uR[j], fuR, P.vR[j], fvR));
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) best = fmax(best, __shfl_xor_sync(FULL, best, off));
    if (lane == 0) atomicMax(key + 1, (unsigned long long)dkey(best));
}

__global__ void k_colsum_partial(int n, int m, const double* __restrict__ Z, double* __restrict__ part)
{
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        double s = 0.0;
        for (int r = r0; r < r1; r++) s += Z[(size_t)r * m + c];
        part[(size_t)blockIdx.x * m + c] = s;
    }
}

__global__ void k_colsum_final(int nb, int m, const double* __restrict__ part, double* __restrict__ out)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += part[(size_t)b * m + c];
    out[c] = s;
}

__global__ void k_gather_subset(int n, int p, ColumnSet cs, const double* __restrict__ X,
                                const double* __restrict__ gall, double* __restrict__ Xs, double* __restrict__ gsub)
{
    const int q = cs.count;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int a = 0; a < q; a++) Xs[(size_t)i * q + a] = X[(size_t)i * p + cs.cols[a]];
    if (i == 0) {
        const int mm = p * (p + 1) / 2, mmq = q * (q + 1) / 2;
        int e = 0;
        for (int a = 0; a < q; a++)
            for (int b = a; b < q; b++) {
                int ca = min(cs.cols[a], cs.cols[b]), cb = max(cs.cols[a], cs.cols[b]);
                gsub[e++] = gall[packed_index(ca, cb, p)];
            }
        for (int a = 0; a < q; a++) gsub[mmq + a] = gall[mm + cs.cols[a]];
    }
}

template <bool GEO>
__global__ void k_tile_far_thr(int n, int tile, const double* __restrict__ thr, double bw, float* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ntiles = (n + tile - 1) / tile;
    if (t >= ntiles) return;
    double rmax = -1.0;
    for (int q = t * tile; q < min(n, (t + 1) * tile); q++) rmax = fmax(rmax, thr ? thr[q] : bw);
    out[t] = tb_far_threshold<GEO>(rmax);
}

}  // namespace

cudaError_t launch_tile_far_thr(int n, int tile, bool geographic, const double* thr, double bw, float* tile_thr,
                                cudaStream_t stream)
{
    const int ntiles = (n + tile - 1) / tile;
    if (geographic)
        k_tile_far_thr<true><<<(ntiles + 255) / 256, 256, 0, stream>>>(n, tile, thr, bw, tile_thr);
    else
        k_tile_far_thr<false><<<(ntiles + 255) / 256, 256, 0, stream>>>(n, tile, thr, bw, tile_thr);
    return cudaGetLastError();
}

cudaError_t launch_column_sums(int n, int m, const double* Z, double* part, int nb, double* out, cudaStream_t stream)
{
    k_colsum_partial<<<nb, 128, 0, stream>>>(n, m, Z, part);
    k_colsum_final<<<(m + 127) / 128, 128, 0, stream>>>(nb, m, part, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_subset(int n, int p, const ColumnSet& cs, const double* X, const double* gall, double* Xs,
                                 double* gsub, cudaStream_t stream)
{
    k_gather_subset<<<(n + 127) / 128, 128, 0, stream>>>(n, p, cs, X, gall, Xs, gsub);
    return cudaGetLastError();
}

cudaError_t launch_build_z(int n, int p, const double* X, const double* y, double* Z, cudaStream_t stream)
{
    k_build_z<<<(n + 127) / 128, 128, 0, stream>>>(n, p, X, y, Z);
    return cudaGetLastError();
}

cudaError_t launch_solve(const SolveArgs& a, int* nblocks, cudaStream_t stream)
{
    if (a.p < 1 || a.p > kMaxP) return cudaErrorInvalidValue;
    if ((a.mode == kSolveAIC || a.mode == kSolveCV) && !a.beta && a.p <= 20) {
        // criterion without beta: one location per thread (k_solve_crit_t)
        const int mm = a.p * (a.p + 1) / 2;
        const size_t smem = (size_t)(mm + 2 * a.p) * ST_THREADS * sizeof(double);
        int grid = (a.n + ST_THREADS - 1) / ST_THREADS;
        if (grid > kSolveMaxBlocks) grid = kSolveMaxBlocks;  // the callers' partials hold this many blocks
        *nblocks = grid;
        if (a.mode == kSolveAIC) {
            raise_smem_limit((const void*)k_solve_crit_t<kSolveAIC>, smem);
            k_solve_crit_t<kSolveAIC><<<grid, ST_THREADS, smem, stream>>>(a);
        } else {
            raise_smem_limit((const void*)k_solve_crit_t<kSolveCV>, smem);
            k_solve_crit_t<kSolveCV><<<grid, ST_THREADS, smem, stream>>>(a);
        }
        return cudaGetLastError();
    }
    int grid = (a.n + SV_WARPS - 1) / SV_WARPS;
    if (grid > kSolveMaxBlocks) grid = kSolveMaxBlocks;
    const int ld = a.p + 1;
    size_t per_warp = (a.mode == kSolveFit) ? 4 * a.p * ld + 2 * a.p : a.p * ld + a.p;
    size_t smem = per_warp * SV_WARPS * sizeof(double);
    *nblocks = grid;
    switch (a.mode) {
    case kSolveAIC:
        raise_smem_limit((const void*)k_solve<kSolveAIC, false>, smem);
        k_solve<kSolveAIC, false><<<grid, SV_WARPS * 32, smem, stream>>>(a, nullptr, nullptr);
        break;
    case kSolveCV:
        raise_smem_limit((const void*)k_solve<kSolveCV, false>, smem);
        k_solve<kSolveCV, false><<<grid, SV_WARPS * 32, smem, stream>>>(a, nullptr, nullptr);
        break;
    case kSolvePredict:
        raise_smem_limit((const void*)k_solve<kSolvePredict, false>, smem);
        k_solve<kSolvePredict, false><<<grid, SV_WARPS * 32, smem, stream>>>(a, nullptr, nullptr);
        break;
    case kSolveRefine:
        raise_smem_limit((const void*)k_solve<kSolveRefine, false>, smem);
        k_solve<kSolveRefine, false><<<grid, SV_WARPS * 32, smem, stream>>>(a, nullptr, nullptr);
        break;
    default:
        raise_smem_limit((const void*)k_solve<kSolveFit, false>, smem);
        k_solve<kSolveFit, false><<<grid, SV_WARPS * 32, smem, stream>>>(a, nullptr, nullptr);
        break;
    }
    return cudaGetLastError();
}

cudaError_t launch_solve_batch(const SolveArgs* segs, const int4* work, int nwork, int mode, int max_p,
                               cudaStream_t stream)
{
    if (max_p < 1 || max_p > kMaxP || nwork < 1 || (mode != kSolveAIC && mode != kSolveCV)) return cudaErrorInvalidValue;
    const size_t smem = (size_t)(max_p * (max_p + 1) + max_p) * SV_WARPS * sizeof(double);
    if (mode == kSolveAIC) {
        raise_smem_limit((const void*)k_solve<kSolveAIC, true>, smem);
        k_solve<kSolveAIC, true><<<nwork, SV_WARPS * 32, smem, stream>>>(SolveArgs{}, segs, work);
    } else {
        raise_smem_limit((const void*)k_solve<kSolveCV, true>, smem);
        k_solve<kSolveCV, true><<<nwork, SV_WARPS * 32, smem, stream>>>(SolveArgs{}, segs, work);
    }
    return cudaGetLastError();
}

// out[4 s + q] = sum of partials[4 b + q] over blocks b in [first[s], first[s + 1]), in order.
__global__ void k_reduce_batch(const double* __restrict__ partials, const int* __restrict__ first,
                               double* __restrict__ out)
{
    const int s = blockIdx.x;
    __shared__ double sh[256][4];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = first[s] + (int)threadIdx.x; b < first[s + 1]; b += 256)
        for (int q = 0; q < 4; q++) acc[q] += partials[b * 4 + q];
    for (int q = 0; q < 4; q++) sh[threadIdx.x][q] = acc[q];
    __syncthreads();
    for (int stride = 128; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride)
            for (int q = 0; q < 4; q++) sh[threadIdx.x][q] += sh[threadIdx.x + stride][q];
        __syncthreads();
    }
    if (threadIdx.x < 4) out[4 * s + threadIdx.x] = sh[0][threadIdx.x];
}

cudaError_t launch_reduce_batch(const double* partials, const int* first, int nseg, double* out, cudaStream_t stream)
{
    k_reduce_batch<<<nseg, 256, 0, stream>>>(partials, first, out);
    return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const double* partials, int nblocks, double* out, cudaStream_t stream)
{
    k_reduce<<<1, 256, 0, stream>>>(partials, nblocks, out);
    return cudaGetLastError();
}

cudaError_t launch_hat_pass(const DevPoints& P, bool geographic, const float4* tb16, const float* tile_thr,
                            const double* X, int p,
                            const double* v, const double* thr, double bw, int kernel, bool skip_tiles,
                            double* qdiag, double* S, int row_target, double* s_row, cudaStream_t stream)
{
    int grid = (P.n + HAT_THREADS - 1) / HAT_THREADS;
    size_t smem = (size_t)(HAT_THREADS + HAT_TILE) * p * sizeof(double);
    if (geographic)
        k_hat<true><<<grid, HAT_THREADS, smem, stream>>>(P, tb16, tile_thr, X, p, v, thr, bw, kernel, skip_tiles ? 1 : 0,
                                                         qdiag, S, row_target, s_row);
    else
        k_hat<false><<<grid, HAT_THREADS, smem, stream>>>(P, tb16, tile_thr, X, p, v, thr, bw, kernel, skip_tiles ? 1 : 0,
                                                          qdiag, S, row_target, s_row);
    return cudaGetLastError();
}

cudaError_t launch_hat_mixed(int n, bool geographic, const float4* pts, const float4* tb16, const float* tile_thr,
                             const double* X, int p, const double* v, const float* thr32, float bw, int kernel,
                             double* qdiag, double* S, int row_target, double* s_row, cudaStream_t stream)
{
    int grid = (n + HAT_THREADS - 1) / HAT_THREADS;
    size_t smem = (size_t)(HAT_THREADS + HAT_TILE) * p * sizeof(float);
    if (geographic)
        k_hat_mixed<true><<<grid, HAT_THREADS, smem, stream>>>(n, pts, tb16, tile_thr, X, p, v, thr32, bw, kernel,
                                                               qdiag, S, row_target, s_row);
    else
        k_hat_mixed<false><<<grid, HAT_THREADS, smem, stream>>>(n, pts, tb16, tile_thr, X, p, v, thr32, bw, kernel,
                                                                qdiag, S, row_target, s_row);
    return cudaGetLastError();
}

cudaError_t launch_max_distance(const DevPoints& P, bool geographic, unsigned long long* key_out, double* rowmax,
                                int num_sms, cudaStream_t stream)
{
    const int grid = num_sms * 8;
    if (geographic) {
        k_maxdist<true><<<grid, 256, 0, stream>>>(P, key_out, rowmax);
        k_maxdist_exact<<<grid, 256, 0, stream>>>(P, key_out, rowmax);
    } else {
        k_maxdist<false><<<grid, 256, 0, stream>>>(P, key_out, rowmax);
    }
    return cudaGetLastError();
}

}  // namespace gwgpu
