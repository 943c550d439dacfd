// k_contract_tc.cu -- mixed-precision W.Z contraction on the tcgen05 tensor cores.
//
// G[i, :] = sum_j w_ij Z~[j, :] for a block of 128 focus rows per CTA:
//  * producer: 256 threads compute the 128 x 32 weight tile of each stage in
//    FP32 from the coordinates (planar or WGS-84 great-circle), split every
//    weight into TF32 hi + lo and store both in the 128-byte-swizzled K-major
//    layout the tensor core reads;
//  * the matching Z~ tile (scaled/centred products, split hi + lo, stored in
//    global memory already in the swizzled image) arrives by one 1-D TMA bulk
//    copy on an mbarrier;
//  * one thread issues 3 x 4 tcgen05.mma.kind::tf32 (hi.hi + hi.lo + lo.hi,
//    K = 8 each) into a 128 x N FP32 accumulator in TMEM and commits to an
//    mbarrier; two stages double-buffer producer and tensor core;
//  * every flush_tiles stages the accumulator is read back with tcgen05.ld
//    and added into double-float (hi, lo) accumulators in global memory, so
//    FP32 rounding never sums more than a chunk of points.
// Compactly supported kernels skip data tiles farther than the block's
// largest threshold (planar boxes).  Waits are bounded and report through err.
#include "gw_common.cuh"
#include "gw_kernels.h"
#include "mixed_weight.cuh"
#include "tc05.cuh"

namespace gwgpu {

namespace {

using namespace tc05;

constexpr int TC_THREADS = 512;
constexpr int TC_M = 128;
constexpr int TC_BK = 32;  // points per stage (128 bytes of TF32 per row)
constexpr uint32_t TC_A_BYTES = TC_M * 128;  // one split part of the weight tile
constexpr uint32_t TC_WAIT = 1u << 22;

struct Smem {
    uint64_t bar_b[2];
    uint64_t bar_mma[2];
    uint64_t bar_p[2];
    uint32_t tmem_base;
    int abort;
};

// Double-float accumulate: (hi, lo) += v.
__device__ __forceinline__ float2 df_add(float2 a, float v)
{
    float s = a.x + v;
    float bp = s - a.x;
    float e = (a.x - (s - bp)) + (v - bp);
    float lo = a.y + e;
    float hi = s + lo;
    return make_float2(hi, lo - (hi - s));
}

// KERN: the weight kernel when fixed at compile time, -1 to read it from the arguments.
template <bool GEO, int KERN>
__global__ void __launch_bounds__(TC_THREADS, 1) k_contract_tc(TcArgs a)
{
    const int kernel = KERN >= 0 ? KERN : a.kernel;
    extern __shared__ unsigned char smem_dyn[];
    __shared__ Smem ctl;
    // 1024-byte aligned stage buffers: [A_hi A_lo B_hi B_lo] x 2
    const uint32_t base_u32 = smem_u32(smem_dyn);
    const uint32_t pad = (1024u - (base_u32 & 1023u)) & 1023u;
    unsigned char* stage0 = smem_dyn + pad;
    const uint32_t b_bytes = (uint32_t)a.npad * 128u;
    const uint32_t stage_bytes = 2u * TC_A_BYTES + 2u * b_bytes;

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int r = t & (TC_M - 1), quarter = t >> 7;
    const int row0 = blockIdx.x * TC_M;
    const int i = row0 + r;
    const bool row_ok = i < a.n;

    if (warp == 0) {
        tmem_alloc(&ctl.tmem_base, 256);
        tmem_relinquish();
    }
    if (t == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(&ctl.bar_b[s], 1);
            mbar_init(&ctl.bar_mma[s], 1);
            mbar_init(&ctl.bar_p[s], 1);
        }
        ctl.abort = 0;
        fence_mbar_init();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = ctl.tmem_base;
    constexpr int NF = GEO ? 2 : 1;                      // float4 per point record
    constexpr uint32_t P_BYTES = NF * 16u * TC_BK;       // point data of one tile

    // focus point
    float4 fa = make_float4(0.f, 0.f, 0.f, 0.f), fb = fa;
    if (row_ok) {
        if (GEO) {
            fa = a.pts[2 * (size_t)i];
            fb = a.pts[2 * (size_t)i + 1];
        } else {
            fa = a.pts[i];
        }
    }
    const float rr = row_ok ? (a.thr ? a.thr[i] : a.bw) : 1.0f;
    const float inv_r2 = 1.0f / (rr * rr);
    // pairs with a haversine term in [s_cut, 0.86] have weight 0 under a compact kernel
    const float s_cut = (GEO && kernel >= GW_KERNEL_BISQUARE) ? geo_s_cut(rr) : __int_as_float(0x7f800000);

    // block bound and largest threshold for tile skipping
    __shared__ float red[TC_THREADS / 32];
    __shared__ float4 fbound_s;
    float rmax = row_ok ? rr : 0.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    if (lane == 0) red[warp] = rmax;
    if (t == 0) fbound_s = tb_union<GEO>(a.tb, row0 / TC_BK, (min(row0 + TC_M, a.n) - 1) / TC_BK);
    __syncthreads();
    rmax = red[0];
    for (int q = 1; q < TC_THREADS / 32; q++) rmax = fmaxf(rmax, red[q]);
    const float4 fbound = fbound_s;
    const float far_thr =
        (a.skip && kernel >= GW_KERNEL_BISQUARE) ? tb_far_threshold<GEO>((double)rmax) : -1.0f;
    // tiles this CTA must visit, one bit per 32-point tile
    uint32_t* tmask = reinterpret_cast<uint32_t*>(stage0 + 2 * (size_t)stage_bytes);
    const int nwords = (a.ntiles + 31) / 32;
    // point data of the current and the next tile (prefetched by TMA)
    float4* ptsbuf = reinterpret_cast<float4*>(stage0 + 2 * (size_t)stage_bytes + (((size_t)nwords * 4 + 15) & ~(size_t)15));
    for (int wd = t; wd < nwords; wd += TC_THREADS) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; b++) {
            const int tile = wd * 32 + b;
            if (tile < a.ntiles && !tb_far<GEO>(fbound, a.tb[tile], far_thr)) bits |= 1u << b;
        }
        tmask[wd] = bits;
    }
    __syncthreads();

    const uint32_t idesc = idesc_tf32(TC_M, a.npad);
    int issued = 0;        // stages issued so far (non-skipped tiles)
    int in_chunk = 0;      // stages accumulated in TMEM since the last flush
    bool first_flush = true;
    bool aborted = false;

    auto flush = [&](int last_stage) {
        // wait for the last MMA group, read TMEM, accumulate in double-float
        const int s = last_stage & 1;
        const uint32_t par = (uint32_t)((last_stage >> 1) & 1);
        if (!mbar_wait(&ctl.bar_mma[s], par, TC_WAIT)) atomicExch(&ctl.abort, 1);
        fence_after_sync();
        const int quad = warp & 3, part = warp >> 2;
        const int lrow = quad * 32 + lane;
        const int grow = row0 + lrow;
        const int ncol_part = a.npad / 4;
        for (int c0 = part * ncol_part; c0 < (part + 1) * ncol_part; c0 += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, v);
            tmem_wait_ld();
            if (grow < a.n) {
                float2* acc = a.acc + (size_t)grow * a.npad + c0;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    float x = __uint_as_float(v[q]);
                    acc[q] = first_flush ? make_float2(x, 0.0f) : df_add(acc[q], x);
                }
            }
        }
        fence_before_sync();
        __syncthreads();
        first_flush = false;
        in_chunk = 0;
    };

    int word = 0;
    uint32_t bits = nwords > 0 ? tmask[0] : 0u;
    auto next_tile = [&]() -> int {
        while (bits == 0 && ++word < nwords) bits = tmask[word];
        if (bits == 0) return -1;
        const int tl = word * 32 + (__ffs(bits) - 1);
        bits &= bits - 1;
        return tl;
    };
    // thread 0 records what it has in flight, for a clean exit after an abort
    int last_b = -1;    // issue index of the last Z copy
    int last_p = -1;    // issue index whose point data was last requested
    int last_mma = -1;  // issue index of the last MMA commit
    int tile = next_tile();
    if (tile >= 0 && t == 0) {
        mbar_arrive_expect_tx(&ctl.bar_p[0], P_BYTES);
        bulk_g2s(ptsbuf, a.pts + (size_t)NF * TC_BK * tile, P_BYTES, &ctl.bar_p[0]);
        last_p = 0;
    }
    while (tile >= 0 && !aborted) {
        const int ntile = next_tile();
        const int s = issued & 1;
        unsigned char* st = stage0 + (size_t)s * stage_bytes;
        unsigned char* A_hi = st;
        unsigned char* A_lo = st + TC_A_BYTES;
        unsigned char* B_hi = st + 2 * TC_A_BYTES;
        if (issued >= 2 && in_chunk >= 2) {
            // the MMAs that read this stage two issues ago must be done
            const uint32_t par = (uint32_t)(((issued >> 1) - 1) & 1);
            if (!mbar_wait(&ctl.bar_mma[s], par, TC_WAIT)) atomicExch(&ctl.abort, 1);
        }
        if (t == 0) {
            mbar_arrive_expect_tx(&ctl.bar_b[s], 2u * b_bytes);
            bulk_g2s(B_hi, a.zimg + (size_t)tile * 2u * b_bytes, 2u * b_bytes, &ctl.bar_b[s]);
            last_b = issued;
            if (ntile >= 0) {
                // the other buffer was last read before the previous iteration's barrier
                mbar_arrive_expect_tx(&ctl.bar_p[s ^ 1], P_BYTES);
                bulk_g2s(ptsbuf + (size_t)(s ^ 1) * NF * TC_BK, a.pts + (size_t)NF * TC_BK * ntile, P_BYTES,
                         &ctl.bar_p[s ^ 1]);
                last_p = issued + 1;
            }
        }
        if (!mbar_wait(&ctl.bar_p[s], (uint32_t)((issued >> 1) & 1), TC_WAIT)) atomicExch(&ctl.abort, 1);
        const float4* tp = ptsbuf + (size_t)s * NF * TC_BK;
        // weight tile: thread (r, quarter) fills points [8*quarter, 8*quarter + 8) of row r
        const int kbase = quarter * 8;
#pragma unroll
        for (int q4 = 0; q4 < 2; q4++) {
            float hi[4], lo[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int k = kbase + q4 * 4 + e;
                const int j = tile * TC_BK + k;
                float w = 0.0f;
                if (row_ok && j < a.n) {
                    float d2 = 0.0f;
                    bool beyond = false;
                    if (GEO) {
                        d2 = geo_d2_32(fa, fb, tp[2 * k], tp[2 * k + 1], s_cut, beyond);
                    } else {
                        d2 = planar_d2_32(fa, tp[k]);
                    }
                    if (!beyond) {
                        w = weight32(kernel, d2, rr, inv_r2);
                        if (a.exclude_self && i == j) w = 0.0f;
                        if (a.wpow == 2) w = w * w;
                    }
                }
                hi[e] = to_tf32(w);
                lo[e] = to_tf32(w - hi[e]);
            }
            const uint32_t off = sw128_offset((uint32_t)r, (uint32_t)(kbase + q4 * 4));
            *reinterpret_cast<float4*>(A_hi + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
            *reinterpret_cast<float4*>(A_lo + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (ctl.abort) {
            aborted = true;
            break;
        }
        if (t == 0) {
            if (!mbar_wait(&ctl.bar_b[s], (uint32_t)((issued >> 1) & 1), TC_WAIT)) {
                atomicExch(&ctl.abort, 1);
            } else {
                fence_after_sync();
                const uint64_t ahi = sw128_kmajor_desc(smem_u32(A_hi));
                const uint64_t alo = sw128_kmajor_desc(smem_u32(A_lo));
                const uint64_t bhi = sw128_kmajor_desc(smem_u32(B_hi));
                const uint64_t blo = sw128_kmajor_desc(smem_u32(B_hi + b_bytes));
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t dk = (uint64_t)(kk * 2);  // 32 bytes = 8 TF32 along K
                    mma_tf32(tmem, ahi + dk, bhi + dk, idesc, (in_chunk > 0 || kk > 0) ? 1u : 0u);
                    mma_tf32(tmem, ahi + dk, blo + dk, idesc, 1u);
                    mma_tf32(tmem, alo + dk, bhi + dk, idesc, 1u);
                }
                mma_commit(&ctl.bar_mma[s]);
                last_mma = issued;
            }
        }
        issued++;
        in_chunk++;
        if (in_chunk >= a.flush_tiles) flush(issued - 1);
        tile = ntile;
    }
    if (!aborted && in_chunk > 0) flush(issued - 1);
    __syncthreads();
    aborted = aborted || ctl.abort;
    // epilogue: double-float -> FP64 rows (only columns of Z)
    if (!aborted) {
        for (int e = t; e < TC_M * a.mcols; e += TC_THREADS) {
            const int lr = e / a.mcols, c = e - lr * a.mcols;
            const int grow = row0 + lr;
            if (grow >= a.n) continue;
            double v = 0.0;
            if (!first_flush) {
                const float2 x = a.acc[(size_t)grow * a.npad + c];
                v = (double)x.x + (double)x.y;
            }
            a.G[(size_t)grow * a.ldg + c] = v;
        }
    } else if (t == 0) {
        atomicExch(a.err, 1);
        // leave no MMA and no bulk copy in flight before TMEM and the CTA go away
        if (last_mma >= 0) mbar_wait(&ctl.bar_mma[last_mma & 1], (uint32_t)((last_mma >> 1) & 1), TC_WAIT);
        if (last_b >= 0) mbar_wait(&ctl.bar_b[last_b & 1], (uint32_t)((last_b >> 1) & 1), TC_WAIT);
        if (last_p >= 0) mbar_wait(&ctl.bar_p[last_p & 1], (uint32_t)((last_p >> 1) & 1), TC_WAIT);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// D[128 x N] = A[128 x 32] * B[N x 32]^T through the same layouts (TF32 in, FP32 out).
__global__ void __launch_bounds__(128, 1) k_tc_selftest(const float* A, const float* B, float* D, int N, int* err)
{
    extern __shared__ unsigned char smem_dyn[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    const uint32_t base_u32 = smem_u32(smem_dyn);
    const uint32_t pad = (1024u - (base_u32 & 1023u)) & 1023u;
    unsigned char* sA = smem_dyn + pad;
    unsigned char* sB = sA + TC_A_BYTES;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    if (warp == 0) {
        tmem_alloc(&tmem_base, 256);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    for (int k = 0; k < 32; k++) *reinterpret_cast<float*>(sA + sw128_offset(t, k)) = to_tf32(A[t * 32 + k]);
    for (int e = t; e < N * 32; e += 128) {
        int row = e / 32, k = e % 32;
        *reinterpret_cast<float*>(sB + sw128_offset(row, k)) = to_tf32(B[row * 32 + k]);
    }
    fence_proxy_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_base;
    if (t == 0) {
        const uint64_t ad = sw128_kmajor_desc(smem_u32(sA)), bd = sw128_kmajor_desc(smem_u32(sB));
        for (int kk = 0; kk < 4; kk++)
            mma_tf32(tmem, ad + (uint64_t)(kk * 2), bd + (uint64_t)(kk * 2), idesc_tf32(128, N), kk > 0 ? 1u : 0u);
        mma_commit(&bar);
    }
    bool ok = mbar_wait(&bar, 0, TC_WAIT);
    fence_after_sync();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            tmem_wait_ld();
            for (int q = 0; q < 16; q++) D[(warp * 32 + lane) * N + c0 + q] = __uint_as_float(v[q]);
        }
    } else {
        atomicExch(err, 1);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// Swizzled Z~ tile images: per 32-point tile, [hi: npad x 128 B][lo: npad x 128 B].
__global__ void k_build_zimg(int n, int mcols, int npad, const double* __restrict__ Z, int ldz,
                             unsigned char* __restrict__ img)
{
    const size_t tile = blockIdx.x;
    const uint32_t b_bytes = (uint32_t)npad * 128u;
    unsigned char* base = img + tile * 2u * b_bytes;
    for (int e = threadIdx.x; e < npad * TC_BK; e += blockDim.x) {
        const int c = e / TC_BK, k = e - c * TC_BK;
        const int j = (int)tile * TC_BK + k;
        const double z = (j < n && c < mcols) ? Z[(size_t)j * ldz + c] : 0.0;
        const float hi = to_tf32((float)z);
        const float lo = to_tf32((float)(z - (double)hi));
        const uint32_t off = sw128_offset((uint32_t)c, (uint32_t)k);
        *reinterpret_cast<float*>(base + off) = hi;
        *reinterpret_cast<float*>(base + b_bytes + off) = lo;
    }
}

}  // namespace

size_t contract_tc_smem_bytes(int npad, int ntiles)
{
    const size_t mask = ((size_t)((ntiles + 31) / 32) * 4 + 15) & ~(size_t)15;
    return 1024 + 2 * (2 * (size_t)TC_A_BYTES + 2 * (size_t)npad * 128) + mask + 2 * 2 * 16 * TC_BK;
}

cudaError_t launch_contract_tc(const TcArgs& a, bool geographic, cudaStream_t stream)
{
    if (a.npad % 64 != 0 || a.npad < 64 || a.npad > 256 || a.mcols > a.npad) return cudaErrorInvalidValue;
    const size_t smem = contract_tc_smem_bytes(a.npad, a.ntiles);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    const int grid = (a.n + TC_M - 1) / TC_M;
    auto go = [&](auto kfn) {
        cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kfn<<<grid, TC_THREADS, smem, stream>>>(a);
    };
    if (geographic) {
        if (a.kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<true, GW_KERNEL_BISQUARE>);
        else if (a.kernel == GW_KERNEL_GAUSSIAN) go(k_contract_tc<true, GW_KERNEL_GAUSSIAN>);
        else go(k_contract_tc<true, -1>);
    } else {
        if (a.kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<false, GW_KERNEL_BISQUARE>);
        else if (a.kernel == GW_KERNEL_GAUSSIAN) go(k_contract_tc<false, GW_KERNEL_GAUSSIAN>);
        else go(k_contract_tc<false, -1>);
    }
    return cudaGetLastError();
}

cudaError_t launch_build_zimg(int n, int mcols, int npad, const double* Z, int ldz, unsigned char* img,
                              cudaStream_t stream)
{
    const int ntiles = (n + TC_BK - 1) / TC_BK;
    k_build_zimg<<<ntiles, 256, 0, stream>>>(n, mcols, npad, Z, ldz, img);
    return cudaGetLastError();
}

cudaError_t launch_tc_selftest(const float* A, const float* B, float* D, int N, int* err, cudaStream_t stream)
{
    if (N % 16 != 0 || N < 16 || N > 256) return cudaErrorInvalidValue;
    const size_t smem = 1024 + TC_A_BYTES + (size_t)N * 128;
    cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_selftest<<<1, 128, smem, stream>>>(A, B, D, N, err);
    return cudaGetLastError();
}

}  // namespace gwgpu
