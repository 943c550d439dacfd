// k_select.cu -- adaptive bandwidth thresholds without sorting.
//
// The reference sorts every distance row to read the b-th smallest distance
// (BandwidthWeight.cpp:40-53 with arma::sort; thrust::sort per row on the
// GPU, BandwidthWeightKernel.cu:71-95).  Here one CTA owns one focus row and
// finds the exact k-th order statistic of the row's FP64 distances with a
// range-bucketed radix select on the IEEE bit pattern (a monotone key):
//   pass 0  histogram of a coarse logarithmic bucket of every key (4096 bins),
//   pass r  histogram of the next bits inside the chosen bucket,
//   gather  once the chosen bucket holds <= 2048 keys, copy them to shared
//           memory and bitonic-sort them there.
// Distances are recomputed in every pass instead of stored, so the kernel
// reads only the coordinates (16-32 B per point, L2 resident).  Integer keys
// make the result bit-exact, ties included.
#include "gw_common.cuh"
#include "gw_kernels.h"

namespace gwgpu {

namespace {

constexpr int SEL_THREADS = 256;
constexpr int SEL_BINS = 4096;
constexpr int SEL_LOG_BINS = 12;
constexpr int SEL_CAP = 2048;
constexpr int SEL_BINS_PER_THREAD = SEL_BINS / SEL_THREADS;

struct SelShared {
    unsigned int hist[SEL_BINS];
    uint64_t cand[SEL_CAP];
    unsigned int warp_tot[SEL_THREADS / 32];
    unsigned int chosen_bin, below, count, ncand;
};

struct Window {
    uint64_t base;  // bucket = (key - base) >> shift, clamped to [0, SEL_BINS)
    int shift;
    uint64_t wlo, whi;  // keys outside [wlo, whi] are ignored
};

__device__ __forceinline__ unsigned bucket_of(const Window& w, uint64_t key)
{
    if (key < w.base) return 0;
    uint64_t q = (key - w.base) >> w.shift;
    return q > (uint64_t)(SEL_BINS - 1) ? (unsigned)(SEL_BINS - 1) : (unsigned)q;
}

__device__ __forceinline__ void bin_range(const Window& w, unsigned b, uint64_t& lo, uint64_t& hi)
{
    lo = (b == 0) ? w.wlo : w.base + ((uint64_t)b << w.shift);
    if (b == SEL_BINS - 1) {
        hi = w.whi;
    } else {
        uint64_t span = ((uint64_t)(b + 1) << w.shift) - 1;
        hi = (span > w.whi - w.base) ? w.whi : w.base + span;
    }
}

// Histogram of the keys of row (fu, fv) inside the window; warp-aggregated
// shared-memory atomics because Morton-adjacent points share bins.
template <bool GEO>
__device__ void hist_pass(SelShared& sh, const DevPoints& P, const Window& w, double fu, double fv, double fuR,
                          double fvR)
{
    for (int b = threadIdx.x; b < SEL_BINS; b += SEL_THREADS) sh.hist[b] = 0;
    __syncthreads();
    const int n = P.n;
    for (int j0 = 0; j0 < n; j0 += SEL_THREADS) {
        int j = j0 + threadIdx.x;
        bool in = false;
        unsigned bin = 0;
        if (j < n) {
            uint64_t key = dkey(pair_dist<GEO>(P, j, fu, fv, fuR, fvR));
            in = key >= w.wlo && key <= w.whi;
            if (in) bin = bucket_of(w, key);
        }
        unsigned act = __ballot_sync(0xffffffffu, in);
        if (in) {
            unsigned peers = __match_any_sync(act, bin);
            int leader = __ffs(peers) - 1;
            if ((int)(threadIdx.x & 31) == leader) atomicAdd(&sh.hist[bin], (unsigned)__popc(peers));
        }
    }
    __syncthreads();
}

// Finds the bin where the cumulative count reaches krem (1-based).
__device__ void scan_pick(SelShared& sh, unsigned krem)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned local = 0;
#pragma unroll
    for (int q = 0; q < SEL_BINS_PER_THREAD; q++) local += sh.hist[t * SEL_BINS_PER_THREAD + q];
    unsigned incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) sh.warp_tot[warp] = incl;
    __syncthreads();
    unsigned wpre = 0;
    for (int q = 0; q < warp; q++) wpre += sh.warp_tot[q];
    unsigned excl = wpre + incl - local;
    if (t == 0) {
        // defaults if no bin reaches krem (cannot happen for a valid rank)
        sh.chosen_bin = SEL_BINS - 1;
        sh.below = 0;
        sh.count = 0;
    }
    __syncthreads();
    if (excl < krem && excl + local >= krem) {
        unsigned c = excl;
        for (int q = 0; q < SEL_BINS_PER_THREAD; q++) {
            unsigned b = t * SEL_BINS_PER_THREAD + q;
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

template <bool GEO>
__device__ void gather_pass(SelShared& sh, const DevPoints& P, uint64_t lo, uint64_t hi, double fu, double fv,
                            double fuR, double fvR)
{
    if (threadIdx.x == 0) sh.ncand = 0;
    __syncthreads();
    const int n = P.n;
    for (int j0 = 0; j0 < n; j0 += SEL_THREADS) {
        int j = j0 + threadIdx.x;
        bool in = false;
        uint64_t key = 0;
        if (j < n) {
            key = dkey(pair_dist<GEO>(P, j, fu, fv, fuR, fvR));
            in = key >= lo && key <= hi;
        }
        unsigned act = __ballot_sync(0xffffffffu, in);
        if (act) {
            int lane = threadIdx.x & 31;
            int leader = __ffs(act) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(&sh.ncand, (unsigned)__popc(act));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (in) {
                unsigned slot = base + __popc(act & ((1u << lane) - 1u));
                if (slot < SEL_CAP) sh.cand[slot] = key;
            }
        }
    }
    __syncthreads();
}

// Ascending bitonic sort of cand[0, len) padded with +inf keys to a power of two.
__device__ void bitonic_sort(SelShared& sh, unsigned count)
{
    unsigned len = 1;
    while (len < count) len <<= 1;
    for (unsigned q = count + threadIdx.x; q < len; q += SEL_THREADS) sh.cand[q] = ~0ull;
    __syncthreads();
    for (unsigned size = 2; size <= len; size <<= 1) {
        for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
            for (unsigned t = threadIdx.x; t < len / 2; t += SEL_THREADS) {
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

template <bool GEO>
__global__ void __launch_bounds__(SEL_THREADS) k_select(DevPoints P, unsigned rank, uint64_t klo, int shift0,
                                                        double* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SelShared& sh = *reinterpret_cast<SelShared*>(smem_raw);
    for (int row = blockIdx.x; row < P.n; row += gridDim.x) {
        const double fu = P.u[row], fv = P.v[row];
        const double fuR = GEO ? P.uR[row] : 0.0, fvR = GEO ? P.vR[row] : 0.0;
        Window w{klo, shift0, 0ull, ~0ull};
        unsigned krem = rank;
        hist_pass<GEO>(sh, P, w, fu, fv, fuR, fvR);
        scan_pick(sh, krem);
        unsigned b = sh.chosen_bin, cnt = sh.count;
        krem -= sh.below;
        uint64_t lo, hi;
        bin_range(w, b, lo, hi);
        __syncthreads();
        while (cnt > (unsigned)SEL_CAP && lo != hi) {
            uint64_t span = hi - lo;
            int bits = 64 - __clzll((long long)span);
            int s = bits > SEL_LOG_BINS ? bits - SEL_LOG_BINS : 0;
            w = Window{lo, s, lo, hi};
            hist_pass<GEO>(sh, P, w, fu, fv, fuR, fvR);
            scan_pick(sh, krem);
            b = sh.chosen_bin;
            cnt = sh.count;
            krem -= sh.below;
            bin_range(w, b, lo, hi);
            __syncthreads();
        }
        double result;
        if (cnt == 0) {
            result = __longlong_as_double(0x7ff8000000000000ll);  // unreachable for 1 <= rank <= n
        } else if (lo == hi) {
            result = keyd(lo);
        } else {
            gather_pass<GEO>(sh, P, lo, hi, fu, fv, fuR, fvR);
            const unsigned nc = min(sh.ncand, (unsigned)SEL_CAP);
            bitonic_sort(sh, nc);
            result = (krem >= 1 && krem <= nc) ? keyd(sh.cand[krem - 1]) : __longlong_as_double(0x7ff8000000000000ll);
        }
        if (threadIdx.x == 0) out[row] = result;
        __syncthreads();
    }
}

// fixbw of BandwidthWeight.cpp:40-53 from the selected order statistics:
// dn < 1: d0 + (d1 - d0) * bx;  dn >= 1: dn * max(dist).
__global__ void k_threshold_combine(int n, double bw, const double* __restrict__ d0,
                                    const double* __restrict__ d1, double* __restrict__ thr)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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

size_t select_smem_bytes() { return sizeof(SelShared); }

cudaError_t launch_select(const DevPoints& P, bool geographic, unsigned rank, double dlo, double dhi,
                          double* out, int num_sms, cudaStream_t stream)
{
    if (rank < 1 || rank > (unsigned)P.n) return cudaErrorInvalidValue;
    // coarse logarithmic window: keys of [dlo, dhi] spread over the 4096 bins
    uint64_t klo, khi;
    {
        uint64_t blo, bhi;
        memcpy(&blo, &dlo, 8);
        memcpy(&bhi, &dhi, 8);
        klo = blo | 0x8000000000000000ull;
        khi = bhi | 0x8000000000000000ull;
    }
    uint64_t span = khi > klo ? khi - klo : 1;
    int bits = 64 - __builtin_clzll(span);
    int shift0 = bits > SEL_LOG_BINS ? bits - SEL_LOG_BINS : 0;
    int grid = num_sms * 6;
    if (grid > P.n) grid = P.n;
    size_t smem = sizeof(SelShared);
    if (geographic) {
        cudaFuncSetAttribute(k_select<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_select<true><<<grid, SEL_THREADS, smem, stream>>>(P, rank, klo, shift0, out);
    } else {
        cudaFuncSetAttribute(k_select<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_select<false><<<grid, SEL_THREADS, smem, stream>>>(P, rank, klo, shift0, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_threshold_combine(int n, double bw, const double* d0, const double* d1, double* thr,
                                     cudaStream_t stream)
{
    k_threshold_combine<<<(n + 255) / 256, 256, 0, stream>>>(n, bw, d0, d1, thr);
    return cudaGetLastError();
}

}  // namespace gwgpu
