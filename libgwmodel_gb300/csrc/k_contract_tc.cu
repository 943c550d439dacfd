// k_contract_tc.cu -- mixed-precision W.Z contraction on the tcgen05 tensor cores.
//
// G[i, :] = sum_j w_ij Z~[j, :] for a block of 128 focus rows per CTA, as a
// warp-specialised pipeline synchronised by mbarriers only:
//  * 16 producer warps compute the 128 x 32 weight tile of each 32-point
//    data tile in FP32 from the point records (planar or WGS-84 great-circle,
//    prefetched into shared memory by a bulk copy two tiles ahead) or from
//    the distance cache, split every weight into TF32 hi + lo and write both
//    into tensor memory (tcgen05.st; five weight stages) or, for npad > 192,
//    into shared memory in the 128-byte-swizzled K-major layout (two stages);
//  * the matching Z~ tile (scaled/centred products, split hi + lo, stored in
//    global memory already in the swizzled image) arrives by 1-D bulk copies
//    issued by one thread of a copy warp, up to four stages ahead (three with
//    weights in shared memory);
//  * one thread of the MMA warp issues 3 x 4 tcgen05.mma.kind::tf32
//    (hi.hi + hi.lo + lo.hi, K = 8 each) per tile, two tiles per pass, into a
//    128 x N FP32 accumulator in TMEM and commits once per tile (tile_done
//    frees both the weight stage and the Z stage of that tile).  An MMA issue returns only when the tensor
//    pipe accepts it (about as long as the MMA runs), so that thread issues
//    nothing else: with the copies on the same thread the pipe idled about
//    two thirds of the time.  Both single-thread loops keep their stage and
//    chunk positions as counters: a division by a run-time value there costs
//    a dependent chain on the thread that gates the whole CTA;
//  * chunks of flush_tiles tiles accumulate in TMEM; four drain warps (one per
//    TMEM lane quadrant) read a finished chunk back with tcgen05.ld and add it
//    into double-float (hi, lo) sums in global memory, so FP32 rounding never
//    sums more than a chunk of points.  With weights in tensor memory there is
//    one accumulator: the drain first copies it out to a staging buffer
//    (coalesced, a few microseconds) and releases it, and adds the staged
//    values while the next chunk runs; otherwise two accumulators alternate.
// Compactly supported kernels skip data tiles farther than the block's
// largest threshold (FP32 tile bounds) and, for great-circle distances, pairs
// beyond the row's haversine cut-off.  Every wait is bounded and reports
// through err.
// With a distance cache (CACHED, geographic) the producers read each pair's
// FP32 squared distance -- filled once per dataset by k_fill_d2_sym with the
// same arithmetic -- instead of computing it: about 14 instead of 58
// instructions per weight, bit-identical weights.  The tile's 16 KB distance
// block takes the place of its point records: a bulk copy np tiles ahead into
// shared memory (after an L2 prefetch nd tiles ahead, both marked evict-first
// in L2), so the producers never wait on global loads.
#include "gw_common.cuh"
#include "gw_kernels.h"
#include "mixed_weight.cuh"
#include "tc05.cuh"

namespace gwgpu {

namespace {

using namespace tc05;

constexpr int TC_PROD_WARPS = 16;
constexpr int TC_PROD = TC_PROD_WARPS * 32;   // producer threads
constexpr int TC_DRAIN_WARPS = 4;             // one per TMEM lane quadrant
constexpr int TC_CTRL_WARP = TC_PROD_WARPS + TC_DRAIN_WARPS;  // issues the MMAs
constexpr int TC_COPY_WARP = TC_CTRL_WARP + 1;                 // issues the Z copies
constexpr int TC_PCOPY_WARP = TC_COPY_WARP + 1;                // issues the point / distance-block copies
constexpr int TC_THREADS = TC_PROD + TC_DRAIN_WARPS * 32 + 96;
constexpr int TC_MAX_NP = 3;  // point / distance-block buffers at most
constexpr int TC_M = 128;
constexpr int TC_BK = 32;  // points per stage (128 bytes of TF32 per row)
constexpr uint32_t TC_A_BYTES = TC_M * 128;  // one split part of the weight tile
constexpr uint32_t TC_WAIT = 1u << 22;
constexpr uint32_t TC_ACC_COLS = 256;  // TMEM column of the second accumulator
// Weights in tensor memory (npad <= 192): one accumulator at column 0 and
// TC_ATM_STAGES weight stages at 192 + 64 s (hi: 32 columns, then lo: 32 columns)
constexpr uint32_t TC_ATM_ACC_COLS = 192;
constexpr uint32_t TC_ATM_A_COL = 192;
constexpr int TC_ATM_STAGES = 5;
constexpr int TC_DONE_SLOTS = 8;  // tile_done slots: tile k commits to slot k % 8
constexpr int TC_MAX_NB = 4;           // Z stages at most
constexpr uint32_t TC_P_MAX = 2u * 16u * TC_BK;  // point records of one tile, geographic
constexpr uint32_t TC_D_BYTES = TC_M * TC_BK * 4;  // one cached 128 x 32 distance block

struct Smem {
    uint64_t full_a[TC_ATM_STAGES];       // weight tile k written: one arrival per producer warp
    uint64_t tile_done[TC_DONE_SLOTS];    // tcgen05.commit after the MMAs of tile k (every earlier MMA too)
    uint64_t full_b[TC_MAX_NB];  // Z tile landed (bulk copy)
    uint64_t full_p[TC_MAX_NP];  // point records or cached distances of a tile landed (bulk copy)
    uint64_t tmem_free[2];       // accumulator drained (read out): one arrival per drain warp
    uint64_t acc_full[2];        // tcgen05.commit after the last MMA of a chunk
    uint32_t tmem_base;
    int abort;
    int ktotal;                  // tiles this CTA visits
    float4 fbound;
    float red[TC_PROD_WARPS];
};

// Walks the tile mask in issue order.
struct TileWalker {
    const uint32_t* mask;
    int nwords, word;
    uint32_t bits;
    __device__ void init(const uint32_t* m, int nw)
    {
        mask = m;
        nwords = nw;
        word = 0;
        bits = nw > 0 ? m[0] : 0u;
    }
    __device__ int next()
    {
        while (bits == 0 && ++word < nwords) bits = mask[word];
        if (bits == 0) return -1;
        const int tl = word * 32 + (__ffs(bits) - 1);
        bits &= bits - 1;
        return tl;
    }
};

// Element (row, col) of the double-float sums and of the staging buffer: rows
// in groups of 128, column-major inside a group, so the 32 lanes of a drain
// warp (32 consecutive rows) touch 32 consecutive elements of one column.
__device__ __forceinline__ size_t acc_at(int row, int col, int npad)
{
    return ((size_t)(row >> 7) * npad + col) * TC_M + (row & (TC_M - 1));
}

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

__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, uint32_t lim)
{
    return __all_sync(0xffffffffu, mbar_wait(bar, parity, lim));
}

// Warp roles: warps 0-15 produce the weight tiles (thread (r, quarter) fills
// points [8 quarter, 8 quarter + 8) of row r); warps 16-19 drain the
// accumulators (warp 16 + q owns TMEM lanes 32 q .. 32 q + 31, all columns);
// lane 0 of warp 20 issues the MMAs and lane 0 of warp 21 the bulk copies
// (Z stage j % nb is refilled once tile_done[j % 8] reports the MMAs of tile j
// done; the same commit frees weight stage j % NW for the producers).  Tile k
// uses weight stage k % NW, Z stage k % nb and point buffer k % 2 (refilled
// once full_a reports the producers done with tile k).  Chunk c = k / F of F
// tiles accumulates in TMEM accumulator c % NACC, whose last MMA commits to
// acc_full; the drain warps read it out and release it through tmem_free.
// Every single-thread wait is for a barrier phase whose successor needs an
// action of that thread still to come, so no waiter can fall two phases behind.
// KERN: the weight kernel when fixed at compile time, -1 to read it from the arguments.
// BATCH: CTA b works on segment work[b].x (arguments segs[work[b].x]) at row
// block work[b].y, so one launch covers many datasets and bandwidths.
// CACHED: weights from the distance cache a.d2c (geographic, single dataset only).
// ATM: the weight tiles live in tensor memory (written with tcgen05.st, read by
// the MMA as its A operand), which frees their 64 KB of shared memory for a
// fourth Z stage and takes their traffic off shared memory; npad <= 192.  With
// one accumulator beside them tensor memory holds five weight stages, so the
// producers run up to five tiles ahead of the MMAs instead of two (the
// producer -> MMA -> producer handshake of two stages left the tensor pipe
// idle about half the time); a.stage must then hold the staging buffer.
template <bool GEO, int KERN, bool BATCH, bool CACHED = false, bool ATM = false>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_contract_tc(TcArgs a0, int nb, int nd, int np, const TcArgs* __restrict__ segs, const int2* __restrict__ work)
{
    static_assert(!CACHED || (GEO && !BATCH), "the distance cache serves single geographic datasets");
    static_assert(!ATM || !BATCH, "tensor-memory weights serve single datasets");
    constexpr uint32_t ACC_COLS = ATM ? TC_ATM_ACC_COLS : TC_ACC_COLS;
    // Weight stages and accumulators.  Tensor memory holds one accumulator and
    // five weight stages (ATM) or two accumulators (weights in shared memory,
    // two stages there).  With one accumulator the MMAs of a chunk wait until
    // the drain warps have copied the previous chunk out of it (a few
    // microseconds per 64 tiles); five stages let the producers run ahead.
    constexpr int NW = ATM ? TC_ATM_STAGES : 2;
    constexpr int NACC = ATM ? 1 : 2;
    const TcArgs a = BATCH ? segs[work[blockIdx.x].x] : a0;
    const int kernel = KERN >= 0 ? KERN : a.kernel;
    // polls of a pipeline wait before it gives up; the waits of the clean-up after
    // a timeout (MMAs and copies in flight) always use TC_WAIT
    const uint32_t lim = a.wait_limit ? a.wait_limit : TC_WAIT;
    extern __shared__ unsigned char smem_dyn[];
    __shared__ Smem ctl;
    const uint32_t base_u32 = smem_u32(smem_dyn);
    const uint32_t pad = (1024u - (base_u32 & 1023u)) & 1023u;
    unsigned char* sA = smem_dyn + pad;  // 2 stages x [A_hi | A_lo]
    const uint32_t b_bytes = (uint32_t)a.npad * 128u;
    unsigned char* sB = sA + (ATM ? 0 : 4 * (size_t)TC_A_BYTES);  // nb stages x [B_hi | B_lo]
    constexpr int NF = GEO ? 2 : 1;                    // float4 per point record
    // per tile: the point records, or with the cache the tile's 128 x 32 distance block
    constexpr uint32_t P_BYTES = CACHED ? TC_D_BYTES : NF * 16u * TC_BK;
    constexpr uint32_t P_SLOT = CACHED ? TC_D_BYTES : TC_P_MAX;  // bytes per buffer (np buffers, np <= NW)
    float4* ptsbuf = reinterpret_cast<float4*>(sB + (size_t)nb * 2 * b_bytes);  // np x P_SLOT
    uint32_t* tmask = reinterpret_cast<uint32_t*>(sB + (size_t)nb * 2 * b_bytes + (size_t)np * P_SLOT);
    const int nwords = (a.ntiles + 31) / 32;

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const long long kstart = (a.prof && t == 0) ? clock64() : 0;
    const bool producer = warp < TC_PROD_WARPS;
    const bool drainer = warp >= TC_PROD_WARPS && warp < TC_CTRL_WARP;
    const int r = t & (TC_M - 1), quarter = (t >> 7) & 3;
    const int row0 = BATCH ? work[blockIdx.x].y : blockIdx.x * TC_M;
    const int i = row0 + r;
    const bool row_ok = producer && i < a.n;

    if (warp == TC_CTRL_WARP) {
        tmem_alloc(&ctl.tmem_base, 512);
        tmem_relinquish();
    }
    if (t == 0) {
        for (int s = 0; s < TC_DONE_SLOTS; s++) mbar_init(&ctl.tile_done[s], 1);
        for (int s = 0; s < NW; s++) mbar_init(&ctl.full_a[s], TC_PROD_WARPS);
        for (int s = 0; s < TC_MAX_NP; s++) mbar_init(&ctl.full_p[s], 1);
        for (int s = 0; s < 2; s++) {
            mbar_init(&ctl.tmem_free[s], TC_DRAIN_WARPS);
            mbar_init(&ctl.acc_full[s], 1);
        }
        for (int s = 0; s < TC_MAX_NB; s++) {
            mbar_init(&ctl.full_b[s], 1);
        }
        ctl.abort = 0;
        fence_mbar_init();
    }
    // focus record
    float4 fa = make_float4(0.f, 0.f, 0.f, 0.f), fb = fa;
    if (row_ok) {
        fa = a.pts[NF * (size_t)i];
        if (GEO) fb = a.pts[2 * (size_t)i + 1];
    }
    const float rr = row_ok ? (a.thr ? a.thr[i] : a.bw) : 1.0f;
    const float inv_r2 = 1.0f / (rr * rr);
    // pairs with a haversine term in [s_cut, 0.86] have weight 0 under a compact kernel
    const float s_cut = (GEO && kernel >= GW_KERNEL_BISQUARE) ? geo_s_cut(rr) : __int_as_float(0x7f800000);
    const int self_j = a.exclude_self ? i : -1;
    // tiles that may hold a self pair of this block's rows (none without exclude_self)
    const int self_t0 = a.exclude_self ? row0 / TC_BK : a.ntiles, self_t1 = (row0 + TC_M - 1) / TC_BK;
    const bool square = a.wpow == 2;

    // block bound and largest threshold for tile skipping
    float rmax = row_ok ? rr : 0.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
    if (producer && lane == 0) ctl.red[warp] = rmax;
    if (t == 0) ctl.fbound = tb_union<GEO>(a.tb, row0 / TC_BK, (min(row0 + TC_M, a.n) - 1) / TC_BK);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = ctl.tmem_base;
    rmax = ctl.red[0];
    for (int q = 1; q < TC_PROD_WARPS; q++) rmax = fmaxf(rmax, ctl.red[q]);
    const float4 fbound = ctl.fbound;
    const float far_thr =
        (a.skip && kernel >= GW_KERNEL_BISQUARE) ? tb_far_threshold<GEO>((double)rmax) : -1.0f;
    // tiles this CTA must visit, one bit per 32-point tile
    for (int wd = t; wd < nwords; wd += TC_THREADS) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; b++) {
            const int tile = wd * 32 + b;
            if (tile < a.ntiles && !tb_far<GEO>(fbound, a.tb[tile], far_thr)) bits |= 1u << b;
        }
        tmask[wd] = bits;
    }
    __syncthreads();
    if (warp == 0) {
        int cnt = 0;
        for (int wd = lane; wd < nwords; wd += 32) cnt += __popc(tmask[wd]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
        if (lane == 0) ctl.ktotal = cnt;
    }
    __syncthreads();
    const int ktotal = ctl.ktotal;

    const int F = a.flush_tiles;
    int k = 0;  // tiles done by this thread's role
    if (producer) {
        TileWalker walk;
        walk.init(tmask, nwords);
        bool ok = true;
        const bool prof = a.prof && t == 0;
        unsigned long long p_stage = 0, p_points = 0, p_weights = 0;  // phase cycles (prof)
        long long c0 = prof ? clock64() : 0, c1 = 0;
        const long long loop0 = c0;
        int ws = 0, pb = 0, ppar = 0;  // k % NW, k % np and (k / np) & 1, kept as counters
        for (int tnext = walk.next(); tnext >= 0; k++) {
            const int tile = tnext;
            tnext = walk.next();
            // another role's timeout: every wait is bounded too, so a look every 16 tiles is enough
            if ((k & 15) == 0 && __any_sync(0xffffffffu, *(volatile int*)&ctl.abort != 0)) {
                ok = false;
                break;
            }
            const int s = ws;
            if (++ws == NW) ws = 0;
            // no self pair and no padding point in this tile: the per-pair checks drop out
            const bool plain = (tile + 1) * TC_BK <= a.n && (self_j < 0 || tile < self_t0 || tile > self_t1);
            if (prof) c0 = clock64();
            // weight stage s is free once the MMAs of tile k - NW are done
            const bool stage_ok = k < NW || warp_wait(&ctl.tile_done[(k - NW) & (TC_DONE_SLOTS - 1)],
                                                      (uint32_t)(((k - NW) >> 3) & 1), lim);
            if (prof) {
                c1 = clock64();
                p_stage += c1 - c0;
                c0 = c1;
            }
            // the tile's point records (or, cached, its distance block) in buffer k % np
            const int pbuf = pb;
            const bool pts_ok = stage_ok && warp_wait(&ctl.full_p[pbuf], (uint32_t)ppar, lim);
            if (++pb == np) {
                pb = 0;
                ppar ^= 1;
            }
            if (!pts_ok) {
                if (lane == 0) atomicExch(&ctl.abort, 1);
                ok = false;
                break;
            }
            if (prof) {
                c1 = clock64();
                p_points += c1 - c0;
                c0 = c1;
            }
            if constexpr (ATM) fence_after_sync();  // the MMAs that read stage s are done
            const float4* tp = ptsbuf + (size_t)pbuf * (P_SLOT / 16);
            unsigned char* A_hi = sA + (size_t)s * 2 * TC_A_BYTES;
            unsigned char* A_lo = A_hi + TC_A_BYTES;
            const int kbase = quarter * 8;
            uint32_t hv[8], lv[8];  // ATM: this thread's 8 columns of the hi and lo tiles
#pragma unroll
            for (int q4 = 0; q4 < 2; q4++) {
                float w[4];
                bool in[4];
                GeoChord g[4];
                if constexpr (CACHED) {
                    // the block is [quarter 4][half 2][row 128][4 points]: row r, points kbase + 4 q4 .. + 3
                    const float4 dv = tp[(2 * quarter + q4) * TC_M + r];
                    const float dd[4] = {dv.x, dv.y, dv.z, dv.w};
                    if (plain) {
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            float v = weight32(kernel, dd[e], rr, inv_r2);
                            v = square ? v * v : v;
                            w[e] = row_ok ? v : 0.0f;
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const int j = tile * TC_BK + kbase + q4 * 4 + e;
                            float v = weight32(kernel, dd[e], rr, inv_r2);
                            v = (j == self_j) ? 0.0f : v;
                            v = square ? v * v : v;
                            w[e] = (row_ok && j < a.n) ? v : 0.0f;
                        }
                    }
                } else {
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int kk = kbase + q4 * 4 + e;
                    in[e] = row_ok && tile * TC_BK + kk < a.n;
                    if (GEO) {
                        g[e] = geo_chord32(fa, fb, tp[2 * kk], tp[2 * kk + 1]);
                        in[e] = in[e] && !geo_beyond(g[e].S, s_cut);
                    }
                    w[e] = 0.0f;
                }
                // the group is skipped only when every lane's four pairs are out
                if (__any_sync(0xffffffffu, in[0] || in[1] || in[2] || in[3])) {
                    // every pair of the warp within 60 degrees: no far-angle branch
                    const bool near = !GEO || __all_sync(0xffffffffu, fmaxf(fmaxf(g[0].S, g[1].S),
                                                                          fmaxf(g[2].S, g[3].S)) <= 0.25f);
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const int kk = kbase + q4 * 4 + e;
                        float d2;
                        if (GEO) d2 = near ? geo_d2_near(g[e]) : geo_d2_far(g[e], fa, fb, tp[2 * kk], tp[2 * kk + 1]);
                        else d2 = planar_d2_32(fa, tp[kk]);
                        float v = weight32(kernel, d2, rr, inv_r2);
                        v = (tile * TC_BK + kk == self_j) ? 0.0f : v;
                        v = square ? v * v : v;
                        w[e] = in[e] ? v : 0.0f;
                    }
                }
                }
                float hi[4], lo[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    hi[e] = to_tf32(w[e]);
                    lo[e] = to_tf32(w[e] - hi[e]);
                }
                if constexpr (ATM) {
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        hv[q4 * 4 + e] = __float_as_uint(hi[e]);
                        lv[q4 * 4 + e] = __float_as_uint(lo[e]);
                    }
                } else {
                    const uint32_t off = sw128_offset((uint32_t)r, (uint32_t)(kbase + q4 * 4));
                    *reinterpret_cast<float4*>(A_hi + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                    *reinterpret_cast<float4*>(A_lo + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
                }
            }
            if constexpr (ATM) {
                // row r is lane r of tensor memory: this warp's lane quadrant is (warp % 4)
                const uint32_t acol = tmem + ((uint32_t)((warp & 3) * 32) << 16) + TC_ATM_A_COL +
                                      (uint32_t)s * 64u + (uint32_t)kbase;
                tmem_st8(acol, hv);
                tmem_st8(acol + 32u, lv);
                tmem_wait_st();
                fence_before_sync();
            } else {
                fence_proxy_async_smem();
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.full_a[s]);
            if (prof) p_weights += clock64() - c0;
        }
        (void)ok;
        if (prof) {
            c1 = clock64();
            atomicAdd(a.prof + kTcProfStageWait, p_stage);
            atomicAdd(a.prof + kTcProfPointsWait, p_points);
            atomicAdd(a.prof + kTcProfWeights, p_weights);
            atomicAdd(a.prof + kTcProfLoop, (unsigned long long)(c1 - loop0));
            atomicAdd(a.prof + kTcProfPrologue, (unsigned long long)(loop0 - kstart));
            atomicMax(a.prof + kTcProfLoopMax, (unsigned long long)(c1 - loop0));
            atomicMax(a.prof + kTcProfTilesMax, (unsigned long long)k);
        }
    } else if (drainer) {
        // chunk c: wait for its last MMA and add the accumulator (this warp's TMEM
        // lane quadrant, every column) into the double-float sums.  Two
        // accumulators: add straight from tensor memory, then release it (the MMAs
        // run on in the other one).  One accumulator: copy it out to the staging
        // buffer first and release it, so the MMAs of the next chunk wait only for
        // that copy, then add the staged values.
        const int quad = warp - TC_PROD_WARPS;
        const int grow = row0 + quad * 32 + lane;
        const int nchunks = (ktotal + F - 1) / F;
        const bool prof = a.prof && lane == 0 && quad == 0;
        unsigned long long pflush = 0;
        const int np = a.npad;
        for (int c = 0; c < nchunks; c++) {
            if (__any_sync(0xffffffffu, *(volatile int*)&ctl.abort != 0)) break;
            const int ab = NACC == 2 ? (c & 1) : 0;
            const uint32_t apar = NACC == 2 ? (uint32_t)((c >> 1) & 1) : (uint32_t)(c & 1);
            if (!warp_wait(&ctl.acc_full[ab], apar, lim)) {
                if (lane == 0) atomicExch(&ctl.abort, 1);
                break;
            }
            const long long c0 = prof ? clock64() : 0;
            fence_after_sync();
            const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)ab * ACC_COLS;
            if constexpr (NACC == 2) {
                for (int col0 = 0; col0 < np; col0 += 16) {
                    uint32_t v[16];
                    tmem_ld16(tbase + (uint32_t)col0, v);
                    tmem_wait_ld();
                    if (grow < a.n) {
                        // the 16 loads first, then the sums: one memory latency per 16 columns
                        float2* __restrict__ e = a.acc + acc_at(grow, col0, np);
                        float2 o[16];
#pragma unroll
                        for (int q = 0; q < 16; q++) o[q] = c == 0 ? make_float2(0.f, 0.f) : e[(size_t)q * TC_M];
#pragma unroll
                        for (int q = 0; q < 16; q++) e[(size_t)q * TC_M] = df_add(o[q], __uint_as_float(v[q]));
                    }
                }
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&ctl.tmem_free[ab]);
            } else {
                for (int col0 = 0; col0 < np; col0 += 32) {
                    uint32_t v0[16], v1[16];
                    const bool two = col0 + 16 < np;  // npad is a multiple of 16
                    tmem_ld16(tbase + (uint32_t)col0, v0);
                    if (two) tmem_ld16(tbase + (uint32_t)col0 + 16u, v1);
                    tmem_wait_ld();
                    if (grow < a.n) {
                        float* st = a.stage + acc_at(grow, col0, np);
#pragma unroll
                        for (int q = 0; q < 16; q++) st[(size_t)q * TC_M] = __uint_as_float(v0[q]);
                        if (two) {
#pragma unroll
                            for (int q = 0; q < 16; q++) st[(size_t)(16 + q) * TC_M] = __uint_as_float(v1[q]);
                        }
                    }
                }
                fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(&ctl.tmem_free[0]);
                if (grow < a.n) {
                    // 16 columns at a time, every load before the sums: one memory
                    // latency per 16 columns
                    for (int col0 = 0; col0 < np; col0 += 16) {
                        const size_t x = acc_at(grow, col0, np);
                        float2* __restrict__ e = a.acc + x;
                        const float* __restrict__ sv = a.stage + x;
                        float2 o[16];
                        float v[16];
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            v[q] = sv[(size_t)q * TC_M];
                            o[q] = c == 0 ? make_float2(0.f, 0.f) : e[(size_t)q * TC_M];
                        }
#pragma unroll
                        for (int q = 0; q < 16; q++) e[(size_t)q * TC_M] = df_add(o[q], v[q]);
                    }
                }
            }
            if (prof) pflush += clock64() - c0;
        }
        if (prof) atomicAdd(a.prof + kTcProfFlush, pflush);
    } else if (warp == TC_CTRL_WARP) {
        // MMA issue (lane 0).  An MMA issue returns only once the tensor pipe takes
        // it, so this thread does nothing but wait for a tile's weights, its Z tile
        // and a free accumulator and issue: every copy is the copy warp's.
        if (lane == 0) {
            int last_mma = -1;
            const uint32_t idesc = idesc_tf32(TC_M, a.npad);
            const bool prof = a.prof != nullptr;
            unsigned long long p_a = 0, p_z = 0, p_i = 0;
            long long c0 = 0, c1 = 0;
            // k % NW, (k / NW) & 1, k % nb, (k / nb) & 1, k % F and k / F kept as
            // counters: divisions by run-time values are long dependent chains on
            // this critical thread
            int ws = 0, wpar = 0, sb = 0, zpar = 0, kf = 0, c = 0;
            // Up to two tiles per pass: the waits for both come first, then their
            // 24 MMAs back to back, so the tensor pipe does not idle through this
            // thread's waits and bookkeeping between the two tiles (2,125 -> 1,843
            // cycles per tile).  Waiting for tile k + 1 before issuing tile k needs
            // its weights (the MMAs of tile k + 1 - NW done) and its Z tile (those
            // of tile k + 1 - nb), both issued already as NW, nb >= 2.  A pass of
            // j tiles needs NW, nb >= j: with two weight stages (weights in shared
            // memory) a longer pass would wait on MMAs it has not issued yet.  A
            // pass never straddles a chunk.
            bool failed = false;
            while (k < ktotal && !failed) {
                if ((k & 15) < 2 && *(volatile int*)&ctl.abort) break;
                const int nt = (k + 1 < ktotal && kf + 1 < F) ? 2 : 1;
                if (prof) c0 = clock64();
                int s2 = ws, wp2 = wpar, sb2 = sb, zp2 = zpar;
                for (int u = 0; u < nt && !failed; u++) {
                    if (!mbar_wait(&ctl.full_a[s2], (uint32_t)wp2, lim) || !mbar_wait(&ctl.full_b[sb2], (uint32_t)zp2, lim))
                        failed = true;
                    if (++s2 == NW) {
                        s2 = 0;
                        wp2 ^= 1;
                    }
                    if (++sb2 == nb) {
                        sb2 = 0;
                        zp2 ^= 1;
                    }
                }
                // a chunk starts once its accumulator is drained (chunk c - NACC)
                if (!failed && kf == 0 && c >= NACC) {
                    bool ok;
                    if constexpr (NACC == 2) ok = mbar_wait(&ctl.tmem_free[c & 1], (uint32_t)(((c >> 1) - 1) & 1), lim);
                    else ok = mbar_wait(&ctl.tmem_free[0], (uint32_t)((c - 1) & 1), lim);
                    failed = !ok;
                }
                if (failed) {
                    atomicExch(&ctl.abort, 1);
                    break;
                }
                if (prof) {
                    c1 = clock64();
                    p_a += c1 - c0;
                    c0 = c1;
                }
                fence_after_sync();
                for (int u = 0; u < nt; u++) {
                    const int s = ws;
                    unsigned char* A_hi = sA + (size_t)s * 2 * TC_A_BYTES;
                    unsigned char* B_hi = sB + (size_t)sb * 2 * b_bytes;
                    const uint64_t ahi = sw128_kmajor_desc(smem_u32(A_hi));
                    const uint64_t alo = sw128_kmajor_desc(smem_u32(A_hi + TC_A_BYTES));
                    const uint64_t bhi = sw128_kmajor_desc(smem_u32(B_hi));
                    const uint64_t blo = sw128_kmajor_desc(smem_u32(B_hi + b_bytes));
                    const uint32_t d = tmem + (NACC == 2 ? (uint32_t)(c & 1) * ACC_COLS : 0u);
                    if constexpr (ATM) {
                        const uint32_t ta = tmem + TC_ATM_A_COL + (uint32_t)s * 64u;  // hi; lo 32 columns on
#pragma unroll
                        for (int kk = 0; kk < 4; kk++) {
                            const uint64_t dk = (uint64_t)(kk * 2);  // 32 bytes = 8 TF32 along K
                            const uint32_t tk = ta + (uint32_t)(kk * 8);
                            mma_tf32_ts(d, tk, bhi + dk, idesc, (kf != 0 || kk > 0) ? 1u : 0u);
                            mma_tf32_ts(d, tk, blo + dk, idesc, 1u);
                            mma_tf32_ts(d, tk + 32u, bhi + dk, idesc, 1u);
                        }
                    } else {
#pragma unroll
                        for (int kk = 0; kk < 4; kk++) {
                            const uint64_t dk = (uint64_t)(kk * 2);  // 32 bytes = 8 TF32 along K
                            mma_tf32(d, ahi + dk, bhi + dk, idesc, (kf != 0 || kk > 0) ? 1u : 0u);
                            mma_tf32(d, ahi + dk, blo + dk, idesc, 1u);
                            mma_tf32(d, alo + dk, bhi + dk, idesc, 1u);
                        }
                    }
                    // one commit frees weight stage s (producers) and Z stage sb (copy warp)
                    mma_commit(&ctl.tile_done[k & (TC_DONE_SLOTS - 1)]);
                    if (kf == F - 1 || k == ktotal - 1) mma_commit(&ctl.acc_full[NACC == 2 ? (c & 1) : 0]);  // chunk c complete
                    last_mma = k;
                    if (++ws == NW) {
                        ws = 0;
                        wpar ^= 1;
                    }
                    if (++sb == nb) {
                        sb = 0;
                        zpar ^= 1;
                    }
                    if (++kf == F) {
                        kf = 0;
                        c++;
                    }
                    k++;
                }
                if (prof) p_i += clock64() - c0;
            }
            if (prof) {
                atomicAdd(a.prof + kTcProfAWait, p_a);
                atomicAdd(a.prof + kTcProfZWait, p_z);
                atomicAdd(a.prof + kTcProfIssue, p_i);
            }
            // leave no MMA in flight before TMEM and the CTA go away
            if (*(volatile int*)&ctl.abort && last_mma >= 0)
                mbar_wait(&ctl.tile_done[last_mma & (TC_DONE_SLOTS - 1)], (uint32_t)((last_mma >> 3) & 1), TC_WAIT);
        }
    } else if (warp == TC_COPY_WARP) {
        // Z copies (lane 0): the Z tiles nb ahead; stage j % nb is refilled once
        // tile_done reports the MMAs of tile j done.  The next phase of that
        // barrier slot (tile j + 8) needs Z tile j + 8, issued only after this
        // wait, so the wait can never be two phases behind.
        if (lane == 0) {
            TileWalker wz;
            wz.init(tmask, nwords);
            int kz = 0;
            int zsb = 0;  // kz % nb, kept as a counter (no run-time divisions on this thread)
            auto issue_z = [&](int tl) {
                const int sb = zsb;
                if (++zsb == nb) zsb = 0;
                unsigned char* B = sB + (size_t)sb * 2 * b_bytes;
                const unsigned char* src = a.zimg + (size_t)tl * 2u * b_bytes;
                mbar_arrive_expect_tx(&ctl.full_b[sb], 2u * b_bytes);
                // four pieces of npad x 64 bytes (multiples of 16): the copy engine overlaps them
                const uint32_t piece = b_bytes / 2;
                for (int q = 0; q < 4; q++) bulk_g2s(B + q * piece, src + q * piece, piece, &ctl.full_b[sb]);
                kz++;
            };
            for (int q = 0; q < nb; q++) {
                const int tl = wz.next();
                if (tl < 0) break;
                issue_z(tl);
            }
            for (int j = 0; j < ktotal && kz < ktotal; j++) {
                if ((j & 15) == 0 && *(volatile int*)&ctl.abort) break;
                if (!mbar_wait(&ctl.tile_done[j & (TC_DONE_SLOTS - 1)], (uint32_t)((j >> 3) & 1), lim)) {
                    atomicExch(&ctl.abort, 1);
                    break;
                }
                const int tl = wz.next();
                if (tl >= 0) issue_z(tl);
            }
            if (*(volatile int*)&ctl.abort) {
                // leave no bulk copy in flight before the CTA goes away
                for (int j = kz - nb > 0 ? kz - nb : 0; j < kz; j++)
                    mbar_wait(&ctl.full_b[j % nb], (uint32_t)((j / nb) & 1), TC_WAIT);
            }
        }
    } else if (warp == TC_PCOPY_WARP) {
        // Point-record copies (lane 0): the records or, with the cache, the 16 KB
        // distance block of a tile np ahead into buffer j % np, once full_a
        // reports the producers done with tile j; with the cache also an L2
        // prefetch of the distance blocks nd ahead.  The next phase of full_a[j %
        // NW] (tile j + NW) needs the copy for tile j + NW, issued after this
        // wait as np <= NW, so the wait can never be two phases behind.
        if (lane == 0) {
            TileWalker wp, wl;
            wp.init(tmask, nwords);
            wl.init(tmask, nwords);
            int kp = 0, kl = 0;  // copies and prefetches issued
            const float* d2blk = CACHED ? a.d2c + (size_t)blockIdx.x * a.ntiles * (TC_D_BYTES / 4) : nullptr;
            // a distance block is read once per launch: first out of L2, so the Z
            // images that every CTA reads stay in it
            const uint64_t stream_pol = l2_policy_evict_first();
            auto issue_l = [&](int tl) {
                bulk_prefetch_l2_hint(d2blk + (size_t)tl * (TC_D_BYTES / 4), TC_D_BYTES, stream_pol);
                kl++;
            };
            int psb = 0;  // kp % np
            auto issue_p = [&](int tl) {
                const int sp = psb;
                if (++psb == np) psb = 0;
                const void* src = CACHED ? static_cast<const void*>(d2blk + (size_t)tl * (TC_D_BYTES / 4))
                                         : static_cast<const void*>(a.pts + (size_t)NF * TC_BK * tl);
                mbar_arrive_expect_tx(&ctl.full_p[sp], P_BYTES);
                if (CACHED) bulk_g2s_hint(ptsbuf + (size_t)sp * (P_SLOT / 16), src, P_BYTES, &ctl.full_p[sp], stream_pol);
                else bulk_g2s(ptsbuf + (size_t)sp * (P_SLOT / 16), src, P_BYTES, &ctl.full_p[sp]);
                kp++;
            };
            for (int q = 0; CACHED && q < nd; q++) {
                const int tl = wl.next();
                if (tl < 0) break;
                issue_l(tl);
            }
            for (int q = 0; q < np; q++) {
                const int tl = wp.next();
                if (tl < 0) break;
                issue_p(tl);
            }
            int pw = 0, wpar = 0;  // j % NW, (j / NW) & 1
            for (int j = 0; j < ktotal && (kp < ktotal || (CACHED && kl < ktotal)); j++) {
                if ((j & 15) == 0 && *(volatile int*)&ctl.abort) break;
                if (CACHED && kl < ktotal) {
                    const int tl = wl.next();
                    if (tl >= 0) issue_l(tl);
                }
                if (kp < ktotal) {
                    if (!mbar_wait(&ctl.full_a[pw], (uint32_t)wpar, lim)) {
                        atomicExch(&ctl.abort, 1);
                        break;
                    }
                    const int tl = wp.next();
                    if (tl >= 0) issue_p(tl);
                }
                if (++pw == NW) {
                    pw = 0;
                    wpar ^= 1;
                }
            }
            if (*(volatile int*)&ctl.abort) {
                for (int j = kp - np > 0 ? kp - np : 0; j < kp; j++)
                    mbar_wait(&ctl.full_p[j % np], (uint32_t)((j / np) & 1), TC_WAIT);
            }
        }
    }
    __syncwarp();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const bool aborted = ctl.abort != 0;
    // epilogue: double-float -> FP64 rows (only columns of Z)
    if (!aborted && producer) {
        const float2* __restrict__ acc = a.acc;
        double* __restrict__ G = a.G;
#pragma unroll 4
        for (int e = t; e < TC_M * a.mcols; e += TC_PROD) {
            const int lr = e / a.mcols, c = e - lr * a.mcols;
            const int grow = row0 + lr;
            if (grow >= a.n) continue;
            double v = 0.0;
            if (k > 0) {
                const float2 x = acc[acc_at(grow, c, a.npad)];
                v = (double)x.x + (double)x.y;
            }
            G[(size_t)grow * a.ldg + c] = v;
        }
    } else if (aborted && t == 0) {
        atomicExch(a.err, 1);
    }
    if (t == 0 && a.tiles && !aborted) atomicAdd(a.tiles, (unsigned long long)k);
    if (t == 0 && a.prof) atomicAdd(a.prof + kTcProfEpilogue, (unsigned long long)(clock64() - kstart));
    fence_before_sync();
    __syncthreads();
    if (warp == TC_CTRL_WARP) tmem_dealloc(tmem, 512);
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

// Symmetric fill of the distance cache.  The FP32 distance is symmetric bit
// for bit (geo_chord32), so each pair of row blocks (A, B), B >= A, is
// computed once: thread (r, q) computes row A * 128 + r against the 32 points
// of tile 4 B + q, writes them as its part of the cache tiles of rows A, and
// keeps them in shared memory, from which the block's transpose becomes the
// cache tiles 4 A .. 4 A + 3 of rows B.  Work items (row block A, chunk of
// FS_CHUNK row blocks B) come from an atomic counter; item_start[A] is the
// first item of row block A.
constexpr int FS_CHUNK = 8;
constexpr int FS_LD = TC_M + 1;  // padded row of the transpose buffer: no bank conflicts either way

__global__ void k_fill_items(int nrb, int* __restrict__ item_start, int* __restrict__ counter)
{
    int acc = 0;
    for (int A = 0; A < nrb; A++) {
        item_start[A] = acc;
        acc += (nrb - A + FS_CHUNK - 1) / FS_CHUNK;
    }
    item_start[nrb] = acc;
    *counter = 0;
}

__global__ void __launch_bounds__(512, 2) k_fill_d2_sym(int n, int ntiles, int nrb, const float4* __restrict__ pts,
                                                         float* __restrict__ d2c,
                                                         const int* __restrict__ item_start, int* __restrict__ counter)
{
    extern __shared__ float sT[];  // 128 x FS_LD: sT[row of A][point of B]
    __shared__ int s_item;
    const int t = threadIdx.x, r = t & (TC_M - 1), q = t >> 7;
    const int nitems = item_start[nrb];
    for (;;) {
        if (t == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= nitems) break;
        int lo = 0, hi = nrb;  // item_start[lo] <= item < item_start[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (item_start[mid] <= item) lo = mid;
            else hi = mid;
        }
        const int A = lo;
        const int B0 = A + (item - item_start[A]) * FS_CHUNK, B1 = min(nrb, B0 + FS_CHUNK);
        const int i = A * TC_M + r;
        float4 fa = make_float4(0.f, 0.f, 0.f, 0.f), fb = fa;
        if (i < n) {
            fa = pts[2 * (size_t)i];
            fb = pts[2 * (size_t)i + 1];
        }
        for (int B = B0; B < B1; B++) {
            const int tile = 4 * B + q;  // warp-uniform
            const bool full = (A + 1) * TC_M <= n && (B + 1) * TC_M <= n;  // no padding row or point
            float4* outA = reinterpret_cast<float4*>(d2c) + ((size_t)A * ntiles + tile) * 1024 + r;
#pragma unroll 2
            for (int g8 = 0; g8 < 8; g8++) {  // points 4 g8 .. 4 g8 + 3 of the tile: [quarter g8 / 2][half g8 % 2]
                float d[4];
                if (tile < ntiles) {
                    GeoChord g[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const size_t j = (size_t)tile * TC_BK + g8 * 4 + e;  // records padded to whole tiles
                        g[e] = geo_chord32(fa, fb, pts[2 * j], pts[2 * j + 1]);
                    }
                    const bool near =
                        __all_sync(0xffffffffu, fmaxf(fmaxf(g[0].S, g[1].S), fmaxf(g[2].S, g[3].S)) <= 0.25f);
                    if (near) {
#pragma unroll
                        for (int e = 0; e < 4; e++) d[e] = geo_d2_near(g[e]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const size_t j = (size_t)tile * TC_BK + g8 * 4 + e;
                            d[e] = geo_d2_far(g[e], fa, fb, pts[2 * j], pts[2 * j + 1]);
                        }
                    }
                    if (!full) {
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const int j = tile * TC_BK + g8 * 4 + e;
                            d[e] = (i < n && j < n) ? d[e] : 3.402823466e38f;
                        }
                    }
                    __stcs(outA + g8 * 128, make_float4(d[0], d[1], d[2], d[3]));
                } else {
                    d[0] = d[1] = d[2] = d[3] = 3.402823466e38f;
                }
                if (B != A) {
#pragma unroll
                    for (int e = 0; e < 4; e++) sT[r * FS_LD + q * TC_BK + g8 * 4 + e] = d[e];
                }
            }
            if (B != A) {
                __syncthreads();
                // rows B * 128 + r against the 32 points of tile 4 A + q: column r of sT
                const int tileA = 4 * A + q;
                if (tileA < ntiles) {
                    float4* outB = reinterpret_cast<float4*>(d2c) + ((size_t)B * ntiles + tileA) * 1024 + r;
#pragma unroll 2
                    for (int g8 = 0; g8 < 8; g8++) {
                        const float* c = sT + (q * TC_BK + g8 * 4) * FS_LD + r;
                        __stcs(outB + g8 * 128, make_float4(c[0], c[FS_LD], c[2 * FS_LD], c[3 * FS_LD]));
                    }
                }
                __syncthreads();
            }
        }
    }
}

}  // namespace

cudaError_t launch_fill_d2_sym(int n, const float4* pts, float* d2c, int* scratch, int num_sms, cudaStream_t stream)
{
    if (n < 1) return cudaErrorInvalidValue;
    const int nrb = (n + TC_M - 1) / TC_M, ntiles = (n + TC_BK - 1) / TC_BK;
    k_fill_items<<<1, 1, 0, stream>>>(nrb, scratch, scratch + nrb + 1);
    const size_t smem = (size_t)TC_M * FS_LD * sizeof(float);
    raise_smem_limit((const void*)k_fill_d2_sym, smem);
    k_fill_d2_sym<<<2 * num_sms, 512, smem, stream>>>(n, ntiles, nrb, pts, d2c, scratch, scratch + nrb + 1);
    return cudaGetLastError();
}

size_t d2_cache_bytes(int n)
{
    const size_t nrb = ((size_t)n + TC_M - 1) / TC_M, ntiles = ((size_t)n + TC_BK - 1) / TC_BK;
    return nrb * ntiles * (size_t)TC_M * TC_BK * sizeof(float);
}


size_t contract_tc_smem_bytes(int npad, int ntiles, int nb, bool cached)
{
    const size_t mask = (size_t)((ntiles + 31) / 32) * 4;
    return 1024 + 4 * (size_t)TC_A_BYTES + (size_t)nb * 2 * npad * 128 + 2 * (size_t)(cached ? TC_D_BYTES : TC_P_MAX) +
           mask;
}

cudaError_t launch_contract_tc(const TcArgs& a, bool geographic, cudaStream_t stream)
{
    if (a.npad % 16 != 0 || a.npad < 16 || a.npad > 256 || a.mcols > a.npad) return cudaErrorInvalidValue;
    if (a.flush_tiles < 2) return cudaErrorInvalidValue;
    const int grid = (a.n + TC_M - 1) / TC_M;
    // cached: the L2 prefetch of the distance blocks runs nd tiles ahead
    const int nd = 4;
    const size_t mask = (size_t)((a.ntiles + 31) / 32) * 4;
    if ((uint32_t)a.npad <= TC_ATM_ACC_COLS) {
        if (!a.stage) return cudaErrorInvalidValue;  // the single accumulator drains through it
        // weights in tensor memory: the shared memory holds only the Z stages and
        // np buffers of point records (or of 16 KB distance blocks with the cache):
        // three when they fit beside four Z stages, else two and fewer Z stages.
        // The barriers' static shared memory comes out of the same 227 KB.
        const size_t pbuf = a.d2c && geographic ? TC_D_BYTES : TC_P_MAX;
        const size_t lim = 227 * 1024 - 1024;
        auto bytes = [&](int b, int p) { return 1024 + (size_t)b * 2 * a.npad * 128 + (size_t)p * pbuf + mask; };
        int nb = TC_MAX_NB, np = TC_MAX_NP;
        if (bytes(nb, np) > lim) np = 2;
        while (nb > 2 && bytes(nb, np) > lim) nb--;
        const size_t smem = bytes(nb, np);
        if (smem > lim) return cudaErrorInvalidValue;
        auto go = [&](auto kfn) {
            raise_smem_limit((const void*)kfn, smem);
            kfn<<<grid, TC_THREADS, smem, stream>>>(a, nb, nd, np, nullptr, nullptr);
        };
        if (geographic && a.d2c) {
            if (a.kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<true, GW_KERNEL_BISQUARE, false, true, true>);
            else if (a.kernel == GW_KERNEL_GAUSSIAN) go(k_contract_tc<true, GW_KERNEL_GAUSSIAN, false, true, true>);
            else go(k_contract_tc<true, -1, false, true, true>);
        } else if (geographic) {
            if (a.kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<true, GW_KERNEL_BISQUARE, false, false, true>);
            else if (a.kernel == GW_KERNEL_GAUSSIAN) go(k_contract_tc<true, GW_KERNEL_GAUSSIAN, false, false, true>);
            else go(k_contract_tc<true, -1, false, false, true>);
        } else {
            if (a.kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<false, GW_KERNEL_BISQUARE, false, false, true>);
            else if (a.kernel == GW_KERNEL_GAUSSIAN) go(k_contract_tc<false, GW_KERNEL_GAUSSIAN, false, false, true>);
            else go(k_contract_tc<false, -1, false, false, true>);
        }
        return cudaGetLastError();
    }
    // wider Z (npad 208 .. 256): weights in shared memory, the kernel read at run time
    int nb = TC_MAX_NB;
    const bool cached = geographic && a.d2c;
    while (nb > 2 && contract_tc_smem_bytes(a.npad, a.ntiles, nb, cached) > 227 * 1024) nb--;
    const size_t smem = contract_tc_smem_bytes(a.npad, a.ntiles, nb, cached);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    auto go = [&](auto kfn) {
        raise_smem_limit((const void*)kfn, smem);
        kfn<<<grid, TC_THREADS, smem, stream>>>(a, nb, nd, 2, nullptr, nullptr);
    };
    if (geographic && a.d2c) go(k_contract_tc<true, -1, false, true>);
    else if (geographic) go(k_contract_tc<true, -1, false>);
    else go(k_contract_tc<false, -1, false>);
    return cudaGetLastError();
}

cudaError_t launch_contract_tc_batch(const TcArgs* segs, const int2* work, int nwork, int max_npad, int max_ntiles,
                                     int flush_tiles, bool geographic, int kernel, cudaStream_t stream)
{
    if (max_npad % 16 != 0 || max_npad < 16 || max_npad > 256 || flush_tiles < 2 || nwork < 1)
        return cudaErrorInvalidValue;
    int nb = TC_MAX_NB;
    while (nb > 2 && contract_tc_smem_bytes(max_npad, max_ntiles, nb, false) > 227 * 1024) nb--;
    const size_t smem = contract_tc_smem_bytes(max_npad, max_ntiles, nb, false);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    TcArgs none{};
    auto go = [&](auto kfn) {
        raise_smem_limit((const void*)kfn, smem);
        kfn<<<nwork, TC_THREADS, smem, stream>>>(none, nb, 2, 2, segs, work);
    };
    if (geographic) {
        if (kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<true, GW_KERNEL_BISQUARE, true>);
        else go(k_contract_tc<true, -1, true>);
    } else {
        if (kernel == GW_KERNEL_BISQUARE) go(k_contract_tc<false, GW_KERNEL_BISQUARE, true>);
        else go(k_contract_tc<false, -1, true>);
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
    raise_smem_limit((const void*)k_tc_selftest, smem);
    k_tc_selftest<<<1, 128, smem, stream>>>(A, B, D, N, err);
    return cudaGetLastError();
}

}  // namespace gwgpu
