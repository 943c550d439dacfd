// k_select.cu -- adaptive bandwidth thresholds without sorting.
//
// The reference sorts every distance row to read the b-th smallest distance
// (BandwidthWeight.cpp:40-53 with arma::sort; thrust::sort per row on the GPU,
// BandwidthWeightKernel.cu:71-95).  Here one CTA of 4 warps owns one focus row
// and finds the k-th order statistic by a range-bucketed radix select:
//
//  * window [T_lo, T_hi]: order statistics of neighbouring ranks computed by
//    earlier golden-section evaluations bracket the answer (0 and +inf when
//    none), so most of the row is classified without looking at points;
//  * tiles of 32 Hilbert-ordered points carry an FP32 bound (planar box or 3-D
//    cap): a tile entirely below T_lo only adds its count, a tile entirely
//    above T_hi is skipped, only straddling tiles are looked at point by point
//    (one point per lane);
//  * a point's FP32 proxy distance carries a proven error band; in the exact
//    (FP64) mode only points whose band meets the window are evaluated with
//    the reference's FP64 formula, so the result is bit-exact, ties included;
//    the mixed mode selects on the proxy itself;
//  * in-window values are histogrammed on their monotone 64-bit keys (4096
//    bins) and gathered into shared memory; once the window holds <= 2048
//    values they are bitonic-sorted there, otherwise the window narrows to
//    the chosen bin and the pass repeats.
#include "gw_common.cuh"
#include "gw_kernels.h"
#include "mixed_weight.cuh"

namespace gwgpu {

namespace {

constexpr int SEL_THREADS = 128;
constexpr int SEL_WARPS = SEL_THREADS / 32;
constexpr int SEL_BINS = 4096;
constexpr int SEL_LOG_BINS = 12;
constexpr int SEL_CAP = 2048;
constexpr int SEL_MAX_PASSES = 10;
constexpr int SEL_TILE = 32;
constexpr int SEL_SEGS = 64;  // coarse segments of the cached histogram (64 bins each)

// Window histogram and candidate buffer of one select CTA.  SelWide (4096
// bins, 2048 candidates) runs passes over whole rows with the logarithmic
// window that the histogram cache also uses; SelNarrow (1024 bins, 1024
// candidates, 12 KB instead of 33 KB of shared memory, so three times the
// CTAs per SM) runs the passes inside one cached bin.
template <int LB_, int CAP_, int THREADS_>
struct SelCfg {
    static constexpr int LB = LB_, BINS = 1 << LB_, CAP = CAP_, THREADS = THREADS_, WARPS = THREADS_ / 32,
                         BPT = BINS / THREADS_;
    struct Shared {
        unsigned int hist[BINS];
        uint64_t cand[CAP];
        unsigned int warp_tot[WARPS];
        unsigned int below_w[WARPS];
        unsigned int chosen_bin, below, count, ncand;
    };
};
using SelWide = SelCfg<SEL_LOG_BINS, SEL_CAP, SEL_THREADS>;
// Inside a cached bin a row's work is mostly a chain of dependent loads
// (segment counts, bins, tile bounds, point records): for small ranks more rows
// in flight per SM (two warps per row, 18 CTAs resident instead of 12) matter
// more than more lanes per row; large ranks walk long rings of tiles, where
// four warps per row are faster.
using SelNarrow = SelCfg<10, 1024, 64>;
using SelNarrow4 = SelCfg<10, 1024, 128>;
constexpr unsigned kNarrow4Rank = 20000;  // ranks above this take four warps per row

struct Window {
    uint64_t base;  // bucket = (key - base) >> shift, clamped to [0, bins)
    int shift;
    uint64_t wlo, whi;  // keys of the window ends (inclusive)
};

template <class C = SelWide>
__device__ __forceinline__ unsigned bucket_of(const Window& w, uint64_t key)
{
    if (key < w.base) return 0;
    uint64_t q = (key - w.base) >> w.shift;
    return q > (uint64_t)(C::BINS - 1) ? (unsigned)(C::BINS - 1) : (unsigned)q;
}

template <class C = SelWide>
__device__ __forceinline__ void bin_range(const Window& w, unsigned b, uint64_t& lo, uint64_t& hi)
{
    lo = (b == 0) ? w.wlo : w.base + ((uint64_t)b << w.shift);
    if (b == C::BINS - 1) {
        hi = w.whi;
    } else {
        uint64_t span = ((uint64_t)(b + 1) << w.shift) - 1;
        hi = (span > w.whi - w.base) ? w.whi : w.base + span;
    }
}

template <class C>
__device__ __forceinline__ Window linear_window(uint64_t lo, uint64_t hi)
{
    uint64_t span = hi - lo;
    int bits = span ? 64 - __clzll((long long)span) : 0;
    return Window{lo, bits > C::LB ? bits - C::LB : 0, lo, hi};
}

// Coarse window over positive distances [dlo, dhi] for whole-row histograms.
__device__ __forceinline__ Window coarse_window(const SelectArgs& a)
{
    const uint64_t klo = (uint64_t)__double_as_longlong(a.dlo) | 0x8000000000000000ull;
    const uint64_t khi = (uint64_t)__double_as_longlong(a.dhi) | 0x8000000000000000ull;
    const uint64_t kspan = khi > klo ? khi - klo : 1;
    const int kbits = 64 - __clzll((long long)kspan);
    const int shift = kbits > SEL_LOG_BINS ? kbits - SEL_LOG_BINS : 0;
    // base aligned to a bin boundary, so a bin is a plain shift of the key
    const uint64_t base = klo & ~((1ull << shift) - 1ull);
    return Window{base, shift, dkey(0.0), dkey(__longlong_as_double(0x7ff0000000000000ll))};
}

// Finds the bin where the cumulative count reaches krem (1-based).
template <class C>
__device__ void scan_pick(typename C::Shared& sh, unsigned krem)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned local = 0;
#pragma unroll
    for (int q = 0; q < C::BPT; q++) local += sh.hist[t * C::BPT + q];
    unsigned incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) sh.warp_tot[warp] = incl;
    if (t == 0) {
        sh.chosen_bin = C::BINS - 1;
        sh.below = 0;
        sh.count = 0;
    }
    __syncthreads();
    unsigned wpre = 0;
    for (int q = 0; q < warp; q++) wpre += sh.warp_tot[q];
    const unsigned excl = wpre + incl - local;
    if (excl < krem && excl + local >= krem) {
        unsigned c = excl;
        for (int q = 0; q < C::BPT; q++) {
            unsigned b = t * C::BPT + q;
            unsigned h = sh.hist[b];
            if (c + h >= krem) {
                sh.chosen_bin = b;
                sh.below = c;
                sh.count = h;
                break;
            }
            c += h;
        }
    }
    __syncthreads();
}

// Ascending bitonic sort of cand[0, count) padded with +inf keys.
template <class C>
__device__ void bitonic_sort(typename C::Shared& sh, unsigned count)
{
    unsigned len = 1;
    while (len < count) len <<= 1;
    for (unsigned q = count + threadIdx.x; q < len; q += C::THREADS) sh.cand[q] = ~0ull;
    __syncthreads();
    for (unsigned size = 2; size <= len; size <<= 1) {
        for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
            for (unsigned t = threadIdx.x; t < len / 2; t += C::THREADS) {
                unsigned i = 2 * t - (t & (stride - 1));
                unsigned j = i + stride;
                bool up = (i & size) == 0;
                uint64_t a = sh.cand[i], b = sh.cand[j];
                if ((a > b) == up) {
                    sh.cand[i] = b;
                    sh.cand[j] = a;
                }
            }
            __syncthreads();
        }
    }
}

struct RowCtx {
    double fu, fv, fuR, fvR;  // FP64 focus coordinates (exact formula)
    float4 fa, fb;            // FP32 proxy record of the focus point
    float qx, qy, qz;         // planar: relative coordinates; geographic: unit vector
};

// Tile classification: -1 entirely below T_lo, +1 entirely above T_hi, 0 straddles.
// Planar thresholds are squared distances, geographic ones 3-D chords.
template <bool GEO>
__device__ __forceinline__ int classify_tile(const float4& tb, const RowCtx& c, float below_thr, float above_thr)
{
    if (GEO) {
        const float dx = tb.x - c.qx, dy = tb.y - c.qy, dz = tb.z - c.qz;
        const float cc = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
        const float hi = (cc + tb.w) * (1.0f + 1e-5f) + 1e-7f;
        const float lo = (cc - tb.w) * (1.0f - 1e-5f) - 1e-7f;
        if (hi < below_thr) return -1;
        if (lo > above_thr && hi < 1.8640781f) return 1;
        return 0;
    } else {
        const float ex = fmaxf(0.0f, fmaxf(tb.x - c.qx, c.qx - tb.y));
        const float ey = fmaxf(0.0f, fmaxf(tb.z - c.qy, c.qy - tb.w));
        const float fx = fmaxf(c.qx - tb.x, tb.y - c.qx);
        const float fy = fmaxf(c.qy - tb.z, tb.w - c.qy);
        const float dmin2 = fmaf(ex, ex, ey * ey) * (1.0f - 1e-5f);
        const float dmax2 = fmaf(fx, fx, fy * fy) * (1.0f + 1e-5f);
        if (dmax2 < below_thr) return -1;
        if (dmin2 > above_thr) return 1;
        return 0;
    }
}

// Runs passes over one row until the rank's value in [T_lo, T_hi] is found.
// EXACT: values are the reference's FP64 distances (proxy band as a filter);
// otherwise the FP32 proxies.  Returns false when the bracket does not hold
// the rank or the pass limit is reached.  The first pass may store its
// histogram (coarse log window over [0, +inf]) in cache_row.
template <bool GEO, bool EXACT, class C>
__device__ bool select_row(typename C::Shared& sh, const SelectArgs& a, const RowCtx& c, double T_lo, double T_hi, Window w,
                           unsigned* cache_row, const float* d2r, double& result)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = a.n;
    const double INF = __longlong_as_double(0x7ff0000000000000ll);
    for (int pass = 0; pass < SEL_MAX_PASSES; pass++) {
        // chord (geographic) or squared-distance (planar) bounds of the window
        // in FP32 with a 1e-5 margin (no FP64 in the per-row work)
        float below_thr, above_thr;
        const float tlo = (float)T_lo, thi = (float)T_hi;
        if (GEO) {
            const float a2 = 2.0f * 6378.137f;
            const float f = 1.0f / 298.257223563f;
            const float wl = tlo / (a2 * (1.0f + f));
            // D <= 2 a w (1 + f) for every half angle w <= pi/2: beyond pi/2 every point is below
            below_thr = !(wl > 0.0f) ? -1.0f : (wl >= 1.5708f ? 1e30f : 2.0f * sinf(wl) * (1.0f - 1e-5f));
            const float wh = thi / (a2 * (1.0f - 2.6f * f));
            above_thr = !(wh < 1.2f) ? 1e30f : 2.0f * sinf(wh) * (1.0f + 1e-5f);
        } else {
            below_thr = tlo > 0.0f ? tlo * tlo * (1.0f - 1e-5f) : -1.0f;
            above_thr = !(thi < 1.8e19f) ? 3e38f : thi * thi * (1.0f + 1e-5f);
        }
        const uint64_t klo = dkey(T_lo), khi = dkey(T_hi);
        for (int b = t; b < C::BINS; b += C::THREADS) sh.hist[b] = 0;
        if (t == 0) sh.ncand = 0;
        __syncthreads();
        unsigned below = 0;
        // each lane classifies one super-tile of 32 tiles (interleaved over the
        // warps, so a row's ring of straddling super-tiles spreads across them);
        // a straddling super-tile is walked tile by tile, a straddling tile
        // point by point
        const int nst = (a.ntiles + 31) / 32;
        for (int sgrp = 0; sgrp * C::WARPS * 32 < nst; sgrp++) {
            const int mys = warp + C::WARPS * (lane + 32 * sgrp);
            int scls = 1;
            if (mys < nst) scls = a.stb ? classify_tile<GEO>(a.stb[mys], c, below_thr, above_thr) : 0;
            if (scls < 0) below += (unsigned)min(32 * SEL_TILE, n - mys * 32 * SEL_TILE);
            unsigned sstr = __ballot_sync(0xffffffffu, scls == 0);
            while (sstr) {
                const int ks = __ffs(sstr) - 1;
                sstr &= sstr - 1;
                const int tbase = (warp + C::WARPS * (ks + 32 * sgrp)) * 32;
                const int mytile = tbase + lane;
                int cls = 1;
                if (mytile < a.ntiles) cls = classify_tile<GEO>(a.tb[mytile], c, below_thr, above_thr);
                if (cls < 0) below += (unsigned)min(SEL_TILE, n - mytile * SEL_TILE);
                unsigned straddle = __ballot_sync(0xffffffffu, cls == 0);
                // with the distance cache, the next straddling tile's value is loaded
                // before this one is used: point `lane` of a tile sits at
                // [quarter lane / 8][half (lane / 4) % 2][row][lane % 4] of its block
                const size_t lane_off = (size_t)(lane >> 2) * 512 + (lane & 3);
                float d2next = 0.0f;
                if (GEO && d2r && straddle) d2next = __ldg(d2r + (size_t)(tbase + __ffs(straddle) - 1) * 4096 + lane_off);
                while (straddle) {
                    const int k = __ffs(straddle) - 1;
                    straddle &= straddle - 1;
                    const int tile = tbase + k;
                    const float d2cached = d2next;
                    if (GEO && d2r && straddle)
                        d2next = __ldg(d2r + (size_t)(tbase + __ffs(straddle) - 1) * 4096 + lane_off);
                    const int j = tile * SEL_TILE + lane;
                    bool in = false;
                    uint64_t key = 0;
                    // the proxy distance of every lane (records are padded to whole tiles),
                    // with the near-angle form when the whole warp is within 60 degrees
                    float d32;
                    if (GEO) {
                        float d2;
                        if (d2r) {
                            d2 = d2cached;  // the same value from the distance cache
                        } else {
                            const float4 pa = a.pts[2 * (size_t)j], pb = a.pts[2 * (size_t)j + 1];
                            const GeoChord g = geo_chord32(c.fa, c.fb, pa, pb);
                            d2 = __all_sync(0xffffffffu, g.S <= 0.25f) ? geo_d2_near(g) : geo_d2_far(g, c.fa, c.fb, pa, pb);
                        }
                        d32 = d2 > 0.0f ? d2 * rsqrt_ftz(d2) : 0.0f;
                    } else {
                        d32 = sqrtf(planar_d2_32(c.fa, a.pts[j]));
                    }
                    if (j < n) {
                        // far-apart pairs (half-angle near pi/2): the FP32 formula is not trusted
                        const bool sure = !GEO || (isfinite(d32) && d32 < 15000.0f);
                        if (EXACT) {
                            double d = (double)d32;
                            const double dl = sure ? d * (1.0 - a.eps) - a.delta : -1.0;
                            const double dh = sure ? d * (1.0 + a.eps) + a.delta : INF;
                            bool eval = false;
                            if (dh < T_lo) below++;
                            else if (!(dl > T_hi)) eval = true;
                            if (eval) {
                                d = pair_dist<GEO>(a.P, j, c.fu, c.fv, c.fuR, c.fvR);
                                if (d < T_lo) below++;
                                else if (d <= T_hi) {
                                    in = true;
                                    key = dkey(d);
                                }
                            }
                        } else if (d32 == d32) {
                            // proxy values compared in key space (dkey is monotone)
                            const uint64_t k32 = dkey_f(d32);
                            if (k32 < klo) below++;
                            else if (k32 <= khi) {
                                in = true;
                                key = k32;
                            }
                        }
                    }
                    const unsigned act = __ballot_sync(0xffffffffu, in);
                    if (act) {
                        if (in) {
                            const unsigned bin = bucket_of<C>(w, key);
                            const unsigned peers = __match_any_sync(act, bin);
                            if (lane == __ffs(peers) - 1) atomicAdd(&sh.hist[bin], (unsigned)__popc(peers));
                        }
                        const int leader = __ffs(act) - 1;
                        unsigned base = 0;
                        if (lane == leader) base = atomicAdd(&sh.ncand, (unsigned)__popc(act));
                        base = __shfl_sync(0xffffffffu, base, leader);
                        if (in) {
                            const unsigned slot = base + __popc(act & ((1u << lane) - 1u));
                            if (slot < C::CAP) sh.cand[slot] = key;
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) below += __shfl_xor_sync(0xffffffffu, below, off);
        if (lane == 0) sh.below_w[warp] = below;
        __syncthreads();
        if constexpr (C::BINS == SEL_BINS) {  // a whole-row pass can fill the cache row
            if (pass == 0 && cache_row)
                for (int b = t; b < SEL_BINS; b += C::THREADS) cache_row[b] = sh.hist[b];
        }
        unsigned below_all = 0;
        for (int q = 0; q < C::WARPS; q++) below_all += sh.below_w[q];
        const unsigned ncand = sh.ncand;
        if (a.rank <= below_all || a.rank > below_all + ncand) {
            __syncthreads();
            return false;
        }
        const unsigned krem = a.rank - below_all;
        if (ncand <= (unsigned)C::CAP) {
            bitonic_sort<C>(sh, ncand);
            result = keyd(sh.cand[krem - 1]);
            __syncthreads();
            return true;
        }
        scan_pick<C>(sh, krem);
        uint64_t lo, hi;
        bin_range<C>(w, sh.chosen_bin, lo, hi);
        __syncthreads();
        if (lo == hi) {
            result = keyd(lo);
            return true;
        }
        T_lo = keyd(lo);
        T_hi = keyd(hi);
        w = linear_window<C>(lo, hi);
    }
    return false;
}

// The adaptive threshold of one row (stage A on the proxies from the cached
// histogram when there is one, stage B on the reference's FP64 values).
template <bool GEO, bool EXACT, class C>
__device__ void select_one(typename C::Shared& sh, const SelectArgs& a, int row, const Window& wlog)
{
    const int t = threadIdx.x;
    const DevPoints P = a.F.u ? a.F : a.P;  // focus coordinates
    const float4* fpts = a.F.u ? a.fpts : a.pts;
    const double INF = __longlong_as_double(0x7ff0000000000000ll);
    RowCtx c;
    c.fu = P.u[row];
    c.fv = P.v[row];
    c.fuR = GEO ? P.uR[row] : 0.0;
    c.fvR = GEO ? P.vR[row] : 0.0;
    if (GEO) {
        c.fa = fpts[2 * (size_t)row];
        c.fb = fpts[2 * (size_t)row + 1];
        c.qx = c.fa.x + c.fb.x;
        c.qy = c.fa.y + c.fb.y;
        c.qz = c.fa.z + c.fb.z;
    } else {
        c.fa = fpts[row];
        c.fb = c.fa;
        c.qx = c.fa.x + c.fa.y;
        c.qy = c.fa.z + c.fa.w;
        c.qz = 0.0f;
    }
    unsigned* cache_row = a.hist_cache ? a.hist_cache + (size_t)row * SEL_BINS : nullptr;
    // stage A: the rank's FP32 proxy value
    double T_lo = 0.0, T_hi = INF;
    Window w = wlog;
    bool ok = true;
    if (cache_row && a.cache_valid) {
        if (a.hist_coarse) {
            // the same bin as scan_pick (the first whose inclusive count reaches the
            // rank) from the row's 64 segment counts and one segment's 64 bins: 512 B
            // of the cache instead of 16 KB, and no block-wide scan
            if (t < 32) {
                const unsigned k = a.rank;
                const unsigned* cp = a.hist_coarse + (size_t)row * SEL_SEGS;
                const unsigned c0 = cp[t], c1 = cp[32 + t];
                const unsigned m0 = __ballot_sync(0xffffffffu, c0 >= k), m1 = __ballot_sync(0xffffffffu, c1 >= k);
                const int seg = m0 ? __ffs(m0) - 1 : (m1 ? 32 + __ffs(m1) - 1 : -1);
                const unsigned prev0 = __shfl_sync(0xffffffffu, c0, (seg - 1) & 31);
                const unsigned prev1 = __shfl_sync(0xffffffffu, c1, (seg - 33) & 31);
                const unsigned base = seg <= 0 ? 0u : (seg <= 32 ? prev0 : prev1);
                unsigned h0 = 0, h1 = 0;
                if (seg >= 0) {
                    h0 = cache_row[seg * 64 + t];
                    h1 = cache_row[seg * 64 + 32 + t];
                }
                unsigned s0 = h0, s1 = h1;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const unsigned v0 = __shfl_up_sync(0xffffffffu, s0, off);
                    const unsigned v1 = __shfl_up_sync(0xffffffffu, s1, off);
                    if (t >= off) {
                        s0 += v0;
                        s1 += v1;
                    }
                }
                s1 += __shfl_sync(0xffffffffu, s0, 31);
                const unsigned f0 = __ballot_sync(0xffffffffu, seg >= 0 && base + s0 >= k);
                const unsigned f1 = __ballot_sync(0xffffffffu, seg >= 0 && base + s1 >= k);
                const int b = f0 ? __ffs(f0) - 1 : (f1 ? 32 + __ffs(f1) - 1 : -1);
                const unsigned hb0 = __shfl_sync(0xffffffffu, h0, b & 31);
                const unsigned hb1 = __shfl_sync(0xffffffffu, h1, b & 31);
                if (t == 0) {
                    if (seg >= 0 && b >= 0) {
                        sh.chosen_bin = (unsigned)(seg * 64 + b);
                        sh.count = b < 32 ? hb0 : hb1;
                    } else {
                        sh.chosen_bin = SEL_BINS - 1;
                        sh.count = 0;
                    }
                }
            }
            __syncthreads();
        } else if constexpr (C::BINS == SEL_BINS) {
            for (int b = t; b < SEL_BINS; b += C::THREADS) sh.hist[b] = cache_row[b];
            __syncthreads();
            scan_pick<C>(sh, a.rank);
        }
        uint64_t lo, hi;
        bin_range<SelWide>(wlog, sh.chosen_bin, lo, hi);
        ok = sh.count > 0;
        __syncthreads();
        T_lo = keyd(lo);
        T_hi = keyd(hi);
        w = linear_window<C>(lo, hi);
        cache_row = nullptr;
    }
    // the row's slice of the distance cache: block row / 128, row row % 128
    const float* d2r =
        GEO && a.d2c && !a.F.u ? a.d2c + (size_t)(row >> 7) * a.ntiles * 4096 + (size_t)(row & 127) * 4 : nullptr;
    double q = __longlong_as_double(0x7ff8000000000000ll);
    if (ok) ok = select_row<GEO, false, C>(sh, a, c, T_lo, T_hi, w, a.cache_valid ? nullptr : cache_row, d2r, q);
    double result = q;
    // stage B: the reference's FP64 value, inside the proxy band around q
    if (EXACT && ok) {
        const double lo = q * (1.0 - a.eps) - a.delta, hi = q * (1.0 + a.eps) + a.delta;
        const double blo = lo > 0.0 ? lo : 0.0;
        ok = select_row<GEO, true, C>(sh, a, c, blo, hi, linear_window<C>(dkey(blo), dkey(hi)), nullptr, d2r, result);
    }
    if (t == 0) {
        if (!ok) {
            atomicMax(a.err, 2);
            result = __longlong_as_double(0x7ff8000000000000ll);
        }
        a.out[row] = result;
    }
    __syncthreads();
}

// C = SelNarrow needs a valid cache with its segment counts (hist_coarse).
template <bool GEO, bool EXACT, class C>
__global__ void __launch_bounds__(C::THREADS) k_select(SelectArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename C::Shared& sh = *reinterpret_cast<typename C::Shared*>(smem_raw);
    // coarse logarithmic window of the first pass over a whole row
    const Window wlog = coarse_window(a);
    const int nrows = a.F.u ? a.F.n : a.n;
    for (int row = blockIdx.x; row < nrows; row += gridDim.x) select_one<GEO, EXACT, C>(sh, a, row, wlog);
}

// Index of the segment holding flattened item `item`: the last seg with start[seg] <= item.
__device__ __forceinline__ int find_segment(const long long* __restrict__ start, int nseg, long long item)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Many selects in one launch: segment s (its own dataset and rank) owns the
// flattened rows [start[s], start[s + 1]).
template <bool GEO, bool EXACT, class C>
__global__ void __launch_bounds__(C::THREADS)
    k_select_batch(const SelectArgs* __restrict__ segs, const long long* __restrict__ start, int nseg)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename C::Shared& sh = *reinterpret_cast<typename C::Shared*>(smem_raw);
    __shared__ SelectArgs sa;
    __shared__ int cur;
    if (threadIdx.x == 0) cur = -1;
    const long long total = start[nseg];
    __syncthreads();
    for (long long item = blockIdx.x; item < total; item += gridDim.x) {
        const int seg = find_segment(start, nseg, item);
        const bool change = seg != cur;  // uniform: cur is stable since the last barrier
        __syncthreads();
        if (change) {
            if (threadIdx.x == 0) {
                sa = segs[seg];
                cur = seg;
            }
            __syncthreads();
        }
        select_one<GEO, EXACT, C>(sh, sa, (int)(item - start[seg]), coarse_window(sa));
    }
}

// Whole-row histograms for the cache: every row's SEL_BINS-bin histogram of
// FP32 proxy distances over the coarse window [dlo, dhi] -- the same counts
// a first select pass over a whole row produces, with the same proxy values.
// HS_ROWS focus rows per CTA share every point record load.  Warp w walks
// groups of 32 tiles; at step q lane l takes point q of tile l, so the 32
// lanes land on points far apart along the curve and rarely hit the same bin.
constexpr int HS_ROWS = 8;
constexpr int HS_THREADS = 1024;  // 32 warps at <= 64 registers: the pass is latency-bound
// Row stride of the shared-memory histograms: one word more than the bins, so
// the same bin of different rows falls in different banks (neighbouring rows
// see nearly the same distances, so their lanes hit the same bins at once).
constexpr int HS_STRIDE = SEL_BINS + 1;

__device__ void hist_store(const unsigned* hs, const SelectArgs& a, int row0, int nrows);

// Histograms of rows [row0, row0 + HS_ROWS) of one dataset into its cache.
template <bool GEO>
__device__ void hist_rows(unsigned* hs, float4 (*rf)[2], const SelectArgs& a, int row0)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = a.n;
    const Window wlog = coarse_window(a);
    constexpr int NF = GEO ? 2 : 1;
    const int ngroups = (a.ntiles + 31) / 32;
    const int nfocus = a.F.u ? a.F.n : n;
    const float4* fpts = a.F.u ? a.fpts : a.pts;
    const int nrows = min(HS_ROWS, nfocus - row0);
    // bucket_of(wlog, dkey_f(d)) for a normal float d in 32/64-bit integer steps:
    // with the aligned base and 29 <= shift <= 52 it is
    // (bits(d) >> (shift - 29)) + (896 << 23 >> (shift - 29)) + (2^63 >> shift) - (base >> shift)
    const bool fastbin = wlog.shift >= 29 && wlog.shift <= 52;
    const int s2 = fastbin ? wlog.shift - 29 : 0;
    const long long kbin = fastbin ? (long long)((896ull << 23) >> s2) + (long long)((1ull << 63) >> wlog.shift) -
                                         (long long)(wlog.base >> wlog.shift)
                                   : 0;
    for (int b = t; b < HS_ROWS * HS_STRIDE; b += HS_THREADS) hs[b] = 0;
    if (t < HS_ROWS * NF) {
        const int r = t / NF, q = t % NF;
        rf[r][q] = r < nrows ? fpts[NF * (size_t)(row0 + r) + q] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    for (int g = warp; g < ngroups; g += HS_THREADS / 32) {
        const int tile = g * 32 + lane;
        for (int q = 0; q < SEL_TILE; q++) {
            const bool valid = tile < a.ntiles && tile * SEL_TILE + q < n;
            const int j = tile < a.ntiles ? tile * SEL_TILE + q : 0;  // records are padded to whole tiles
            const float4 pa = a.pts[NF * (size_t)j];
            const float4 pb = GEO ? a.pts[2 * (size_t)j + 1] : pa;
            // one row at a time (its record from shared memory), so the registers
            // stay within the 64 that 32 warps per SM leave; the near-angle form
            // is voted per row (it equals the general form wherever S <= 0.25)
#pragma unroll
            for (int r = 0; r < HS_ROWS; r++) {
                const float4 ra = rf[r][0];
                float d32;
                if (GEO) {
                    const float4 rb = rf[r][1];
                    const GeoChord gc = geo_chord32(ra, rb, pa, pb);
                    const bool near = __all_sync(0xffffffffu, gc.S <= 0.25f);
                    const float d2 = near ? geo_d2_near(gc) : geo_d2_far(gc, ra, rb, pa, pb);
                    d32 = d2 > 0.0f ? d2 * rsqrt_ftz(d2) : 0.0f;
                } else {
                    d32 = sqrtf(planar_d2_32(ra, pa));
                }
                if (!valid || r >= nrows) continue;
                if (d32 == d32) {
                    const uint32_t fb = __float_as_uint(d32);
                    unsigned bin;
                    if (fastbin) {
                        const long long q = (long long)(fb >> s2) + kbin;
                        bin = fb < 0x00800000u ? 0u : (unsigned)min(max(q, 0ll), (long long)(SEL_BINS - 1));
                    } else {
                        bin = bucket_of(wlog, dkey_f(d32));
                    }
                    atomicAdd(&hs[r * HS_STRIDE + bin], 1u);
                }
            }
        }
    }
    __syncthreads();
    hist_store(hs, a, row0, nrows);
}

// Writes the histograms of rows [row0, row0 + nrows) into the cache, with
// their cumulative segment counts.
__device__ void hist_store(const unsigned* hs, const SelectArgs& a, int row0, int nrows)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int e = t; e < nrows * SEL_BINS; e += HS_THREADS)
        a.hist_cache[(size_t)row0 * SEL_BINS + e] = hs[(e / SEL_BINS) * HS_STRIDE + e % SEL_BINS];
    if (a.hist_coarse) {
        // cumulative counts at the end of every 64-bin segment: one warp per row
        for (int r = warp; r < nrows; r += HS_THREADS / 32) {
            const unsigned* hr = hs + r * HS_STRIDE;
            unsigned s0 = 0, s1 = 0;
            for (int b = 0; b < 64; b++) {  // rotated start: the 32 lanes hit 32 different banks
                const int q = (b + lane) & 63;
                s0 += hr[lane * 64 + q];
                s1 += hr[(32 + lane) * 64 + q];
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned v0 = __shfl_up_sync(0xffffffffu, s0, off);
                const unsigned v1 = __shfl_up_sync(0xffffffffu, s1, off);
                if (lane >= off) {
                    s0 += v0;
                    s1 += v1;
                }
            }
            s1 += __shfl_sync(0xffffffffu, s0, 31);
            unsigned* cp = a.hist_coarse + (size_t)(row0 + r) * SEL_SEGS;
            cp[lane] = s0;
            cp[32 + lane] = s1;
        }
    }
    __syncthreads();
}

// Whole-row histograms read back from a filled distance cache a.d2c (layout
// of launch_fill_d2_sym): the same proxy values, so the same counts as
// hist_rows.  Lane (r = lane % 8, u = lane / 8) of warp w reads all 32
// values of row row0 + r in tile w + 32 (4 s + u), s = 0, 1, ...: each warp
// load is four whole 128-byte lines, all 32 values are loaded before the
// first is used (the pass streams the whole cache), and the 32 lanes of one
// shared-memory atomic are 8 rows x 4 tiles far apart along the curve, which
// rarely hit the same bin.
__device__ void hist_rows_cached(unsigned* hs, const SelectArgs& a, int row0)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n = a.n;
    const Window wlog = coarse_window(a);
    const bool fastbin = wlog.shift >= 29 && wlog.shift <= 52;
    const int s2 = fastbin ? wlog.shift - 29 : 0;
    const long long kbin = fastbin ? (long long)((896ull << 23) >> s2) + (long long)((1ull << 63) >> wlog.shift) -
                                         (long long)(wlog.base >> wlog.shift)
                                   : 0;
    const bool bin32 = fastbin && kbin > -(1ll << 30) && kbin + (long long)(0x7f800000u >> s2) < (1ll << 30);
    const int kbin32 = bin32 ? (int)kbin : 0;
    const int nrows = min(HS_ROWS, n - row0);
    for (int b = t; b < HS_ROWS * HS_STRIDE; b += HS_THREADS) hs[b] = 0;
    __syncthreads();
    const int r = lane & 7, u = lane >> 3;
    const int row = row0 + r;
    const bool row_ok = r < nrows;
    unsigned* hrow = hs + r * HS_STRIDE;
    const float4* in = reinterpret_cast<const float4*>(a.d2c) + (size_t)(row / 128) * a.ntiles * 1024 + (row & 127);
    constexpr int WARPS = HS_THREADS / 32;
    // the bin of one value; values that are not points (padding, rows past n) and
    // NaN go to word SEL_BINS of the row, the padding word that is never stored.
    // The window's form is fixed for the pass, so each form has its own loop.
    auto pass = [&](auto bin_of) {
        for (int base = 0; base < a.ntiles; base += 4 * WARPS) {
            const int tile = base + 4 * warp + u;
            const bool tile_ok = tile < a.ntiles;
            float4 dv[8];  // [quarter][half]: points 4 k .. 4 k + 3 of the tile
#pragma unroll
            for (int k = 0; k < 8; k++)
                dv[k] = tile_ok ? __ldcs(in + (size_t)tile * 1024 + k * 128) : make_float4(0.f, 0.f, 0.f, 0.f);
            const int nv = (row_ok && tile_ok) ? min(SEL_TILE, n - tile * SEL_TILE) : 0;  // points of the 32
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const float d[4] = {dv[k].x, dv[k].y, dv[k].z, dv[k].w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float d32 = d[e] > 0.0f ? d[e] * rsqrt_ftz(d[e]) : 0.0f;
                    const unsigned bin = (k * 4 + e < nv && d32 == d32) ? bin_of(d32) : (unsigned)SEL_BINS;
                    atomicAdd(&hrow[bin], 1u);
                }
            }
        }
    };
    if (bin32) {
        pass([&](float d32) {
            const uint32_t fb = __float_as_uint(d32);
            const int qb = (int)(fb >> s2) + kbin32;
            return fb < 0x00800000u ? 0u : (unsigned)min(max(qb, 0), SEL_BINS - 1);
        });
    } else if (fastbin) {
        pass([&](float d32) {
            const uint32_t fb = __float_as_uint(d32);
            const long long qb = (long long)(fb >> s2) + kbin;
            return fb < 0x00800000u ? 0u : (unsigned)min(max(qb, 0ll), (long long)(SEL_BINS - 1));
        });
    } else {
        pass([&](float d32) { return bucket_of(wlog, dkey_f(d32)); });
    }
    __syncthreads();
    hist_store(hs, a, row0, nrows);
}

__global__ void __launch_bounds__(HS_THREADS, 1) k_select_hist_cached(SelectArgs a)
{
    extern __shared__ __align__(16) unsigned hs[];  // HS_ROWS x HS_STRIDE
    for (int row0 = blockIdx.x * HS_ROWS; row0 < a.n; row0 += gridDim.x * HS_ROWS) hist_rows_cached(hs, a, row0);
}

template <bool GEO>
__global__ void __launch_bounds__(HS_THREADS, 1) k_select_hist(SelectArgs a)
{
    extern __shared__ __align__(16) unsigned hs[];  // HS_ROWS x HS_STRIDE
    __shared__ float4 rf[HS_ROWS][2];
    const int nfocus = a.F.u ? a.F.n : a.n;
    for (int row0 = blockIdx.x * HS_ROWS; row0 < nfocus; row0 += gridDim.x * HS_ROWS) hist_rows<GEO>(hs, rf, a, row0);
}

// Histogram caches of many datasets in one launch: segment s owns the row
// groups [start[s], start[s + 1]) of HS_ROWS rows each.
template <bool GEO>
__global__ void __launch_bounds__(HS_THREADS, 1)
    k_select_hist_batch(const SelectArgs* __restrict__ segs, const long long* __restrict__ start, int nseg)
{
    extern __shared__ __align__(16) unsigned hs[];
    __shared__ float4 rf[HS_ROWS][2];
    __shared__ SelectArgs sa;
    __shared__ int cur;
    if (threadIdx.x == 0) cur = -1;
    __syncthreads();
    const long long total = start[nseg];
    for (long long item = blockIdx.x; item < total; item += gridDim.x) {
        const int seg = find_segment(start, nseg, item);
        const bool change = seg != cur;
        __syncthreads();
        if (change) {
            if (threadIdx.x == 0) {
                sa = segs[seg];
                cur = seg;
            }
            __syncthreads();
        }
        hist_rows<GEO>(hs, rf, sa, (int)(item - start[seg]) * HS_ROWS);
    }
}

// thr[i] = (float)v[i] over the flattened rows of many segments.
__global__ void k_to_float_batch(const double* const* __restrict__ in, float* const* __restrict__ out,
                                 const long long* __restrict__ start, int nseg)
{
    const long long total = start[nseg];
    for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < total;
         item += (long long)gridDim.x * blockDim.x) {
        const int seg = find_segment(start, nseg, item);
        const long long i = item - start[seg];
        out[seg][i] = (float)in[seg][i];
    }
}

// fixbw of BandwidthWeight.cpp:40-53 from the selected order statistics:
// dn < 1: d0 + (d1 - d0) * bx;  dn >= 1: dn * max(dist).
__global__ void k_threshold_combine(int rows, int n, double bw, const double* __restrict__ d0,
                                    const double* __restrict__ d1, double* __restrict__ thr)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    double dn = bw / n;
    if (dn < 1) {
        double b0 = floor(bw), bx = bw - b0;
        double a = d0[i], c = d1 ? d1[i] : a;
        thr[i] = a + (c - a) * bx;
    } else {
        thr[i] = dn * d0[i];
    }
}

__global__ void k_to_float(int n, const double* __restrict__ in, float* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

}  // namespace

cudaError_t launch_to_float(int n, const double* in, float* out, cudaStream_t stream)
{
    k_to_float<<<(n + 255) / 256, 256, 0, stream>>>(n, in, out);
    return cudaGetLastError();
}

size_t select_smem_bytes() { return sizeof(SelWide::Shared); }

template <class C>
cudaError_t launch_select_cfg(const SelectArgs& a, bool geographic, bool exact, int grid, cudaStream_t stream)
{
    const size_t smem = sizeof(typename C::Shared);
#define GW_SEL(G, E)                                                          \
    do {                                                                      \
        raise_smem_limit((const void*)k_select<G, E, C>, smem);               \
        k_select<G, E, C><<<grid, C::THREADS, smem, stream>>>(a);             \
    } while (0)
    if (geographic) {
        if (exact) GW_SEL(true, true);
        else GW_SEL(true, false);
    } else {
        if (exact) GW_SEL(false, true);
        else GW_SEL(false, false);
    }
#undef GW_SEL
    return cudaGetLastError();
}

cudaError_t launch_select(const SelectArgs& a, bool geographic, bool exact, int num_sms, cudaStream_t stream)
{
    if (a.rank < 1 || a.rank > (unsigned)a.n) return cudaErrorInvalidValue;
    const int nrows = a.F.u ? a.F.n : a.n;
    // inside a cached bin the small window buffers fit three times the CTAs per SM
    const bool narrow = a.hist_cache && a.cache_valid && a.hist_coarse;
    const bool wide_rows = a.rank > kNarrow4Rank;
    int grid = num_sms * (narrow ? (wide_rows ? 32 : 48) : 12);
    if (grid > nrows) grid = nrows;
    if (!narrow) return launch_select_cfg<SelWide>(a, geographic, exact, grid, stream);
    return wide_rows ? launch_select_cfg<SelNarrow4>(a, geographic, exact, grid, stream)
                     : launch_select_cfg<SelNarrow>(a, geographic, exact, grid, stream);
}

cudaError_t launch_select_hist_cached(const SelectArgs& a, int num_sms, cudaStream_t stream)
{
    if (!a.hist_cache || !a.d2c || a.F.u || a.n < 1) return cudaErrorInvalidValue;
    const size_t smem = (size_t)HS_ROWS * HS_STRIDE * sizeof(unsigned);
    int grid = (a.n + HS_ROWS - 1) / HS_ROWS;
    if (grid > num_sms) grid = num_sms;
    raise_smem_limit((const void*)k_select_hist_cached, smem);
    k_select_hist_cached<<<grid, HS_THREADS, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_select_hist(const SelectArgs& a, bool geographic, int num_sms, cudaStream_t stream)
{
    if (!a.hist_cache || a.n < 1) return cudaErrorInvalidValue;
    const size_t smem = (size_t)HS_ROWS * HS_STRIDE * sizeof(unsigned);
    int grid = (a.n + HS_ROWS - 1) / HS_ROWS;
    if (grid > num_sms) grid = num_sms;
    if (geographic) {
        raise_smem_limit((const void*)k_select_hist<true>, smem);
        k_select_hist<true><<<grid, HS_THREADS, smem, stream>>>(a);
    } else {
        raise_smem_limit((const void*)k_select_hist<false>, smem);
        k_select_hist<false><<<grid, HS_THREADS, smem, stream>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_select_hist_batch(const SelectArgs* segs, const long long* start, int nseg, bool geographic,
                                     int num_sms, cudaStream_t stream)
{
    const size_t smem = (size_t)HS_ROWS * HS_STRIDE * sizeof(unsigned);
    if (geographic) {
        raise_smem_limit((const void*)k_select_hist_batch<true>, smem);
        k_select_hist_batch<true><<<num_sms, HS_THREADS, smem, stream>>>(segs, start, nseg);
    } else {
        raise_smem_limit((const void*)k_select_hist_batch<false>, smem);
        k_select_hist_batch<false><<<num_sms, HS_THREADS, smem, stream>>>(segs, start, nseg);
    }
    return cudaGetLastError();
}

cudaError_t launch_select_batch(const SelectArgs* segs, const long long* start, int nseg, bool geographic, bool exact,
                                int num_sms, cudaStream_t stream)
{
    // every segment carries a valid cache with its segment counts: the narrow window buffers
    const int grid = num_sms * 36;
    const size_t smem = sizeof(SelNarrow::Shared);
#define GW_SELB(G, E)                                                                                       \
    do {                                                                                                    \
        raise_smem_limit((const void*)k_select_batch<G, E, SelNarrow>, smem);                               \
        k_select_batch<G, E, SelNarrow><<<grid, SelNarrow::THREADS, smem, stream>>>(segs, start, nseg);     \
    } while (0)
    if (geographic) {
        if (exact) GW_SELB(true, true);
        else GW_SELB(true, false);
    } else {
        if (exact) GW_SELB(false, true);
        else GW_SELB(false, false);
    }
#undef GW_SELB
    return cudaGetLastError();
}

cudaError_t launch_to_float_batch(const double* const* in, float* const* out, const long long* start, int nseg,
                                  int num_sms, cudaStream_t stream)
{
    k_to_float_batch<<<num_sms * 4, 256, 0, stream>>>(in, out, start, nseg);
    return cudaGetLastError();
}

cudaError_t launch_threshold_combine(int n, double bw, const double* d0, const double* d1, double* thr,
                                     cudaStream_t stream)
{
    return launch_threshold_combine_rows(n, n, bw, d0, d1, thr, stream);
}

cudaError_t launch_threshold_combine_rows(int rows, int n, double bw, const double* d0, const double* d1, double* thr,
                                          cudaStream_t stream)
{
    k_threshold_combine<<<(rows + 255) / 256, 256, 0, stream>>>(rows, n, bw, d0, d1, thr);
    return cudaGetLastError();
}

}  // namespace gwgpu
