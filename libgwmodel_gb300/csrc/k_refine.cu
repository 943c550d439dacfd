// k_refine.cu -- iterative refinement of the mixed-precision local solves.
//
// The tensor-core contraction gives A~_i and b~_i to about 1e-6 relative; the
// Cholesky solve of A~_i beta = b~_i inherits that error times cond(A_i).  One
// refinement step computes the residual of the local normal equation directly
// from the data,
//     r_i = sum_j w_ij x~_j (y~_j - x~_j^T beta_i),
// with the very FP32 weights the contraction used, and then solves
// A~_i delta = r_i with the existing factor (k_solve's refine mode).  The
// residual is ~1e-5 of its terms (it is what the first solve missed) and
// e_ij = y~_j - x~_j^T beta_i cancels an order of magnitude, so the products
// and sums run in double-float arithmetic: FP32 pairs (hi, lo) with
// error-free products (fma) and sums (TwoSum), ~44 bits, about five times
// faster than FP64 on a GPU whose FP64 rate is 1/64 of FP32.
// One thread owns one focus row; data tiles beyond the block's largest
// threshold are skipped exactly as in the contraction.  With the distance
// cache the 128 rows of a CTA are one row block of the cache, so a tile's
// squared distances are read coalesced instead of recomputed (the same FP32
// values the contraction weighted).
#include "gw_common.cuh"
#include "gw_kernels.h"
#include "mixed_weight.cuh"

namespace gwgpu {

namespace {

constexpr int RF_THREADS = 128;
constexpr int RF_TILE = 32;

// Double-float value hi + lo, |lo| <= ulp(hi) / 2.
struct DF {
    float h, l;
};

__device__ __forceinline__ DF df_of(double x)
{
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}

// Dekker's FastTwoSum (|a| >= |b| or a == 0).
__device__ __forceinline__ DF df_fast(float a, float b)
{
    const float s = a + b;
    return DF{s, b - (s - a)};
}

// a + b: Knuth's TwoSum of the high parts, then the low parts folded in.
__device__ __forceinline__ DF df_add(DF a, DF b)
{
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb);
    return df_fast(s, e + (a.l + b.l));
}

// a * b with the exact product of the high parts (one fma).
__device__ __forceinline__ DF df_mul(DF a, DF b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast(p, e);
}

// a * w for a single float w.
__device__ __forceinline__ DF df_mul_f(DF a, float w)
{
    const float p = a.h * w;
    return df_fast(p, fmaf(a.l, w, fmaf(a.h, w, -p)));
}

template <bool GEO, int PMAX>
__global__ void __launch_bounds__(RF_THREADS) k_refine(RefineArgs a)
{
    extern __shared__ DF rsm[];  // RF_TILE x (p + 1): x~_j then y~_j, double-float
    __shared__ float4 fbound_s;
    __shared__ float red[RF_THREADS / 32];
    const int p = a.p, pp = a.p + 1;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int row0 = blockIdx.x * RF_THREADS;
    const int i = row0 + t;
    const bool ok = i < a.n;

    float4 fa = make_float4(0.f, 0.f, 0.f, 0.f), fb = fa;
    if (ok) {
        if (GEO) {
            fa = a.pts[2 * (size_t)i];
            fb = a.pts[2 * (size_t)i + 1];
        } else {
            fa = a.pts[i];
        }
    }
    const float rr = ok ? (a.thr ? a.thr[i] : a.bw) : 1.0f;
    const float inv_r2 = 1.0f / (rr * rr);
    DF beta[PMAX], r[PMAX];
#pragma unroll
    for (int k = 0; k < PMAX; k++) {
        beta[k] = df_of((ok && k < p) ? a.beta[(size_t)i * p + k] : 0.0);
        r[k] = DF{0.0f, 0.0f};
    }
    float rmax = ok ? rr : 0.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    if (lane == 0) red[warp] = rmax;
    if (t == 0) fbound_s = tb_union<GEO>(a.tb, row0 / RF_TILE, (min(row0 + RF_THREADS, a.n) - 1) / RF_TILE);
    __syncthreads();
    rmax = red[0];
    for (int q = 1; q < RF_THREADS / 32; q++) rmax = fmaxf(rmax, red[q]);
    const float4 fbound = fbound_s;
    const float far_thr =
        (a.skip && a.kernel >= GW_KERNEL_BISQUARE) ? tb_far_threshold<GEO>((double)rmax) : -1.0f;
    // this thread's elements of a tile's staging block (point q, column c), once:
    // no division by the run-time p + 1 inside the tile loop
    constexpr int RF_LOADS = (RF_TILE * (PMAX + 1) + RF_THREADS - 1) / RF_THREADS;
    int lq[RF_LOADS], lc[RF_LOADS];
#pragma unroll
    for (int u = 0; u < RF_LOADS; u++) {
        const int e = t + u * RF_THREADS;
        lq[u] = e / pp;
        lc[u] = e - lq[u] * pp;
    }

    // cache block (row block, tile): [quarter 4][half 2][row 128][4 points], so point q of
    // this thread's row is component q % 4 of float4 (q / 4) * 128 + row
    static_assert(RF_THREADS == 128 && RF_TILE == 32, "one CTA is one row block of the distance cache");
    const float* d2base = (GEO && a.d2c) ? a.d2c + (size_t)blockIdx.x * a.ntiles * 4096 + 4 * t : nullptr;
    for (int tile = 0; tile < a.ntiles; tile++) {
        if (tb_far<GEO>(fbound, a.tb[tile], far_thr)) continue;
        const int j0 = tile * RF_TILE;
#pragma unroll
        for (int u = 0; u < RF_LOADS; u++) {
            const int e = t + u * RF_THREADS;
            if (e < RF_TILE * pp) {
                const int j = j0 + lq[u], c = lc[u];
                rsm[e] = df_of((j < a.n) ? (c < p ? a.X[(size_t)j * p + c] : a.y[j]) : 0.0);
            }
        }
        __syncthreads();
        if (ok) {
            const int qend = min(RF_TILE, a.n - j0);
            for (int q = 0; q < qend; q++) {
                const float w = d2base ? weight32(a.kernel, d2base[(size_t)tile * 4096 + (q >> 2) * 512 + (q & 3)], rr,
                                                  inv_r2)
                                       : mixed_weight<GEO>(a.pts, j0 + q, fa, fb, a.kernel, rr, inv_r2);
                if (w == 0.0f) continue;
                const DF* xj = rsm + q * pp;
                DF e = xj[p];
#pragma unroll
                for (int k = 0; k < PMAX; k++) {
                    if (k < p) {
                        const DF m = df_mul(xj[k], beta[k]);
                        e = df_add(e, DF{-m.h, -m.l});
                    }
                }
                const DF we = df_mul_f(e, w);
#pragma unroll
                for (int k = 0; k < PMAX; k++)
                    if (k < p) r[k] = df_add(r[k], df_mul(we, xj[k]));
            }
        }
        __syncthreads();
    }
    if (ok)
        for (int k = 0; k < p; k++) a.r[(size_t)i * p + k] = (double)r[k].h + (double)r[k].l;
}

template <bool GEO, int PMAX>
cudaError_t launch_pm(const RefineArgs& a, cudaStream_t s)
{
    const int grid = (a.n + RF_THREADS - 1) / RF_THREADS;
    const size_t smem = (size_t)RF_TILE * (a.p + 1) * sizeof(DF);
    k_refine<GEO, PMAX><<<grid, RF_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

// The unrolled loops run PMAX iterations predicated on k < p, and every
// predicated-off instruction still takes its issue slot: the bound follows p
// in steps of two (one above 16).
template <bool GEO>
cudaError_t launch_geo(const RefineArgs& a, cudaStream_t s)
{
    switch (a.p) {
    case 1: case 2: return launch_pm<GEO, 2>(a, s);
    case 3: case 4: return launch_pm<GEO, 4>(a, s);
    case 5: case 6: return launch_pm<GEO, 6>(a, s);
    case 7: case 8: return launch_pm<GEO, 8>(a, s);
    case 9: case 10: return launch_pm<GEO, 10>(a, s);
    case 11: case 12: return launch_pm<GEO, 12>(a, s);
    case 13: case 14: return launch_pm<GEO, 14>(a, s);
    case 15: case 16: return launch_pm<GEO, 16>(a, s);
    case 17: return launch_pm<GEO, 17>(a, s);
    case 18: return launch_pm<GEO, 18>(a, s);
    case 19: return launch_pm<GEO, 19>(a, s);
    case 20: return launch_pm<GEO, 20>(a, s);
    case 21: return launch_pm<GEO, 21>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_refine_residual(const RefineArgs& a, bool geographic, cudaStream_t stream)
{
    return geographic ? launch_geo<true>(a, stream) : launch_geo<false>(a, stream);
}

}  // namespace gwgpu
