// engine.cpp -- host side of the device-resident GWR engine.
#include "engine.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <thread>

#include "gw_kernels.h"
#include "golden.h"

namespace gwgpu {

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

// Position of cell (x, y) along the Hilbert curve over a 2^31 x 2^31 grid
// (Hilbert's space-filling curve, by the usual quadrant rotate-and-reflect
// recursion from the top bit down).  Unlike the Z-order curve it never jumps:
// consecutive cells are neighbours, so any run of consecutive points is
// spatially compact.
uint64_t hilbert_index(uint32_t x, uint32_t y)
{
    const uint32_t n = 1u << 31;
    uint64_t d = 0;
    for (uint32_t s = n >> 1; s > 0; s >>= 1) {
        const uint32_t rx = (x & s) ? 1u : 0u;
        const uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = n - 1 - x;
                y = n - 1 - y;
            }
            const uint32_t tmp = x;
            x = y;
            y = tmp;
        }
    }
    return d;
}

// fn(begin, end) over [0, n) in contiguous chunks on the host's threads (at
// least `grain` items per chunk); the calling thread takes the first chunk.
template <class F>
void parallel_for(size_t n, size_t grain, F&& fn)
{
    const size_t T = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), 64));
    const size_t chunks = std::min(T, (n + grain - 1) / std::max<size_t>(grain, 1));
    if (chunks <= 1) {
        fn((size_t)0, n);
        return;
    }
    const size_t step = (n + chunks - 1) / chunks;
    std::vector<std::thread> pool;
    for (size_t c = 1; c < chunks; c++) {
        const size_t b = c * step, e = std::min(n, b + step);
        if (b < e) pool.emplace_back([&fn, b, e] { fn(b, e); });
    }
    fn((size_t)0, std::min(n, step));
    for (auto& t : pool) t.join();
}

// Stable LSD radix sort of (key, index) pairs by key, 8 bits a pass (passes
// whose byte is the same for every key are skipped): for input in index
// order, the same permutation std::sort gives the pairs.
void radix_sort(std::vector<std::pair<uint64_t, int>>& a)
{
    const size_t n = a.size();
    std::vector<std::pair<uint64_t, int>> b(n);
    uint64_t all_or = 0, all_and = ~0ull;
    for (const auto& x : a) {
        all_or |= x.first;
        all_and &= x.first;
    }
    for (int shift = 0; shift < 64; shift += 8) {
        if ((((all_or ^ all_and) >> shift) & 0xff) == 0) continue;
        size_t cnt[257] = {};
        for (const auto& x : a) cnt[((x.first >> shift) & 0xff) + 1]++;
        for (int q = 0; q < 256; q++) cnt[q + 1] += cnt[q];
        for (const auto& x : a) b[cnt[(x.first >> shift) & 0xff]++] = x;
        a.swap(b);
    }
}

// FP64 unit vectors (cos lat cos lon, cos lat sin lon, sin lat) of points given
// in radians, as three arrays of n: the chord form of the great-circle
// distance, and the source of every geographic record and bound below.
std::vector<double> unit_vectors(const std::vector<double>& lonR, const std::vector<double>& latR)
{
    const size_t n = lonR.size();
    std::vector<double> e(3 * n);
    parallel_for(n, 4096, [&](size_t b, size_t en) {
        for (size_t s = b; s < en; s++) {
            const double cl = std::cos(latR[s]);
            e[s] = cl * std::cos(lonR[s]);
            e[n + s] = cl * std::sin(lonR[s]);
            e[2 * n + s] = std::sin(latR[s]);
        }
    });
    return e;
}

// Geographic bounds of consecutive tiles of `size` points (sorted order), from
// the points' unit vectors (3 x n).
std::vector<TileCap> make_caps(const std::vector<double>& e, int size)
{
    const int n = (int)(e.size() / 3), nt = (n + size - 1) / size;
    std::vector<TileCap> caps(nt);
    parallel_for((size_t)nt, 256, [&](size_t tb, size_t te) {
        for (int t = (int)tb; t < (int)te; t++) {
            const int s0 = t * size, s1 = std::min(n, s0 + size);
            double sx = 0, sy = 0, sz = 0;
            for (int s = s0; s < s1; s++) {
                sx += e[s];
                sy += e[(size_t)n + s];
                sz += e[2 * (size_t)n + s];
            }
            double nrm = std::sqrt(sx * sx + sy * sy + sz * sz);
            TileCap c{1.0, 0.0, 0.0, 2.0};  // degenerate tile: no bound
            if (nrm > 1e-12) {
                c = TileCap{sx / nrm, sy / nrm, sz / nrm, 0.0};
                for (int s = s0; s < s1; s++) {
                    const double dx = e[s] - c.cx, dy = e[(size_t)n + s] - c.cy, dz = e[2 * (size_t)n + s] - c.cz;
                    c.rho = std::max(c.rho, std::sqrt(dx * dx + dy * dy + dz * dz));
                }
                c.rho = c.rho * (1.0 + 1e-12) + 1e-15;
            }
            caps[t] = c;
        }
    });
    return caps;
}

void split_fp32(double v, float& hi, float& lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// FP32 records of the points (hu, hv), padded to whole 32-point tiles: planar
// (u - uc, v - vc) split hi/lo in one float4; geographic the unit vector split
// hi/lo in two float4 (its z is sin(lat)).
// e: the points' unit vectors (3 x n), geographic only.
std::vector<float4> point_records(const std::vector<double>& hu, const std::vector<double>& hv, bool geographic,
                                  double uc, double vc, const std::vector<double>& e)
{
    const int n = (int)hu.size();
    const size_t nt32 = (size_t)(n + 31) / 32;
    std::vector<float4> pts;
    if (!geographic) {
        pts.assign(nt32 * 32, make_float4(0.f, 0.f, 0.f, 0.f));
        parallel_for((size_t)n, 8192, [&](size_t b, size_t en) {
            for (size_t s = b; s < en; s++) {
                float a, bb, c, d;
                split_fp32(hu[s] - uc, a, bb);
                split_fp32(hv[s] - vc, c, d);
                pts[s] = make_float4(a, bb, c, d);
            }
        });
    } else {
        pts.assign(2 * nt32 * 32, make_float4(0.f, 0.f, 0.f, 0.f));
        parallel_for((size_t)n, 8192, [&](size_t b, size_t en) {
            for (size_t s = b; s < en; s++) {
                float xh, xl, yh, yl, zh, zl;
                split_fp32(e[s], xh, xl);
                split_fp32(e[(size_t)n + s], yh, yl);
                split_fp32(e[2 * (size_t)n + s], zh, zl);
                pts[2 * s] = make_float4(xh, yh, zh, 0.f);
                pts[2 * s + 1] = make_float4(xl, yl, zl, 0.f);
            }
        });
    }
    return pts;
}

// FP32 bounds of consecutive tiles of `size` points, rounded outward: planar
// boxes relative to (uc, vc) widened by `slack`, geographic 3-D caps.

std::vector<float4> tile_bounds(const std::vector<double>& hu, const std::vector<double>& hv, bool geographic,
                                int size, double uc, double vc, double slack, const std::vector<double>& e)
{
    const int n = (int)hu.size();
    const int nt = (n + size - 1) / size;
    std::vector<float4> tb(nt);
    if (!geographic) {
        for (int t = 0; t < nt; t++) {
            double ulo = hu[t * size], uhi = ulo, vlo = hv[t * size], vhi = vlo;
            for (int s = t * size; s < std::min(n, (t + 1) * size); s++) {
                ulo = std::min(ulo, hu[s]);
                uhi = std::max(uhi, hu[s]);
                vlo = std::min(vlo, hv[s]);
                vhi = std::max(vhi, hv[s]);
            }
            tb[t] = make_float4(nextafterf((float)(ulo - uc - slack), -INFINITY),
                                nextafterf((float)(uhi - uc + slack), INFINITY),
                                nextafterf((float)(vlo - vc - slack), -INFINITY),
                                nextafterf((float)(vhi - vc + slack), INFINITY));
        }
    } else {
        std::vector<TileCap> cp = make_caps(e, size);
        for (int t = 0; t < nt; t++)
            tb[t] = make_float4((float)cp[t].cx, (float)cp[t].cy, (float)cp[t].cz,
                                nextafterf((float)cp[t].rho, INFINITY) * (1.0f + 1e-6f) + 1e-7f);
    }
    return tb;
}

// GWRBase::AICc (GWRBase.h:90-94) from RSS and tr(S).
double aicc(double n, double rss, double trS)
{
    return n * std::log(rss / n) + n * std::log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
}

// The distance cache of each device, shared by the engines on it (see
// Engine::setDistanceCacheLimit).  Every launch that fills or reads it runs
// under `mu` and records `used` on its engine's stream; a new owner's stream
// waits for that event before it overwrites the buffer.
struct DeviceD2Cache {
    std::mutex mu;
    float* ptr = nullptr;
    size_t bytes = 0;
    const Engine* owner = nullptr;
    cudaEvent_t used = nullptr;
};
constexpr int kMaxDevices = 64;
// Allocated once and never destroyed, so engines that outlive static
// destruction at process exit still find their device's entry and mutex.
DeviceD2Cache* const g_d2c = new DeviceD2Cache[kMaxDevices];

DeviceD2Cache& device_d2c(int device)
{
    if (device < 0 || device >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
    return g_d2c[device];
}

// Frees the device's cache (the caller holds its lock); waits for its last use.
void free_d2c(DeviceD2Cache& c)
{
    if (c.used) cudaEventSynchronize(c.used);
    if (c.ptr) cudaFree(c.ptr);
    c.ptr = nullptr;
    c.bytes = 0;
    c.owner = nullptr;
}

}  // namespace

Engine::Engine(int device) : device_(device)
{
    check(cudaSetDevice(device), "cudaSetDevice");
    cudaDeviceProp prop;
    check(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    num_sms_ = prop.multiProcessorCount;
    check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    check(cudaMallocHost(&host_sums_, 8 * sizeof(double)), "cudaMallocHost");
}

Engine::~Engine()
{
    if (stream_) cudaStreamSynchronize(stream_);
    if (device_ >= 0 && device_ < kMaxDevices) {
        DeviceD2Cache& c = g_d2c[device_];
        std::lock_guard<std::mutex> lk(c.mu);
        if (c.owner == this) {
            cudaSetDevice(device_);
            free_d2c(c);
        }
    }
    for (auto& e : events_)
        if (e) cudaEventDestroy(e);
    for (auto& pt : pending_) {
        cudaEventDestroy(pt.e0);
        cudaEventDestroy(pt.e1);
    }
    if (host_sums_) cudaFreeHost(host_sums_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Engine::synchronize() { check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize"); }

DevPoints Engine::points() const
{
    DevPoints P;
    P.n = n_;
    P.u = u_.get();
    P.v = v_.get();
    P.uR = uR_.get();
    P.vR = vR_.get();
    P.e = e_.get();
    return P;
}


void Engine::setData(int n, int p, const double* x, const double* y, const double* coords, bool geographic)
{
    if (n < 2) throw std::invalid_argument("GWRBasic needs at least two data points");
    if (p < 1 || p > kMaxP) throw std::invalid_argument("number of independent variables must be in [1, 32]");
    check(cudaSetDevice(device_), "cudaSetDevice");
    n_ = n;
    p_ = p;
    mm_ = p * (p + 1) / 2;
    m_ = mm_ + p;
    geographic_ = geographic;
    thr_valid_ = false;
    gall_valid_ = false;
    mixed_ready_ = false;

    // Hilbert order of the coordinates
    double umin = coords[0], umax = coords[0], vmin = coords[n], vmax = coords[n];
    for (int i = 0; i < n; i++) {
        umin = std::min(umin, coords[i]);
        umax = std::max(umax, coords[i]);
        vmin = std::min(vmin, coords[n + i]);
        vmax = std::max(vmax, coords[n + i]);
    }
    const double su = umax > umin ? 2147483647.0 / (umax - umin) : 0.0;
    const double sv = vmax > vmin ? 2147483647.0 / (vmax - vmin) : 0.0;
    std::vector<std::pair<uint64_t, int>> keyed(n);
    parallel_for((size_t)n, 4096, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) {
            double fu = (coords[i] - umin) * su, fv = (coords[n + i] - vmin) * sv;
            uint32_t qu = std::isfinite(fu) ? (uint32_t)std::min(std::max(fu, 0.0), 2147483647.0) : 0u;
            uint32_t qv = std::isfinite(fv) ? (uint32_t)std::min(std::max(fv, 0.0), 2147483647.0) : 0u;
            keyed[i] = {hilbert_index(qu, qv), (int)i};
        }
    });
    radix_sort(keyed);
    perm_.resize(n);
    for (int s = 0; s < n; s++) perm_[s] = keyed[s].second;

    std::vector<double> hu(n), hv(n), huR, hvR, hx((size_t)n * p), hy(n);
    const double DE2RA = M_PI / 180;
    if (geographic) {
        huR.resize(n);
        hvR.resize(n);
    }
    parallel_for((size_t)n, 4096, [&](size_t b, size_t e) {
        for (size_t s = b; s < e; s++) {
            const int i = perm_[s];
            hu[s] = coords[i];
            hv[s] = coords[n + i];
            if (geographic) {
                huR[s] = hu[s] * DE2RA;
                hvR[s] = hv[s] * DE2RA;
            }
            for (int k = 0; k < p; k++) hx[s * p + k] = x[(size_t)i + (size_t)k * n];
            hy[s] = y[i];
        }
    });
    const int ntiles = (n + kTile - 1) / kTile;
    std::vector<TileBox> ht(ntiles);
    for (int t = 0; t < ntiles; t++) {
        TileBox b{hu[t * kTile], hu[t * kTile], hv[t * kTile], hv[t * kTile]};
        for (int s = t * kTile; s < std::min(n, (t + 1) * kTile); s++) {
            b.ulo = std::min(b.ulo, hu[s]);
            b.uhi = std::max(b.uhi, hu[s]);
            b.vlo = std::min(b.vlo, hv[s]);
            b.vhi = std::max(b.vhi, hv[s]);
        }
        ht[t] = b;
    }
    if (geographic) {
        dhi_ = 20300.0;  // above half the WGS-84 meridian circumference with the flattening term
    } else {
        double du = umax - umin, dv = vmax - vmin;
        dhi_ = std::sqrt(du * du + dv * dv) * (1.0 + 1e-9);
        if (!(dhi_ > 0.0) || !std::isfinite(dhi_)) dhi_ = 1.0;
    }
    dlo_ = std::ldexp(dhi_, -24);

    u_.alloc(n);
    v_.alloc(n);
    if (geographic) {
        uR_.alloc(n);
        vR_.alloc(n);
    } else {
        uR_.clear();
        vR_.clear();
    }
    x_.alloc((size_t)n * p);
    y_.alloc(n);
    z_.alloc((size_t)n * m_);
    g_.alloc((size_t)n * m_);
    thr_.alloc(n);
    sel0_.alloc(n);
    sel1_.alloc(n);
    beta_.alloc((size_t)n * p);
    sii_.alloc(n);
    resid_.alloc(n);
    partials_.alloc(4096 * 4);
    sums_.alloc(8);
    tiles_.alloc(ntiles);
    key_.alloc(2);
    check(cudaMemcpyAsync(u_.get(), hu.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D u");
    check(cudaMemcpyAsync(v_.get(), hv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D v");
    if (geographic) {
        check(cudaMemcpyAsync(uR_.get(), huR.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D");
        check(cudaMemcpyAsync(vR_.get(), hvR.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D");
        he_ = unit_vectors(huR, hvR);
        e_.alloc(he_.size());
        check(cudaMemcpyAsync(e_.get(), he_.data(), sizeof(double) * he_.size(), cudaMemcpyHostToDevice, stream_),
              "H2D unit vectors");
    } else {
        he_.clear();
        e_.clear();
    }
    check(cudaMemcpyAsync(x_.get(), hx.data(), sizeof(double) * hx.size(), cudaMemcpyHostToDevice, stream_),
          "H2D x");
    check(cudaMemcpyAsync(y_.get(), hy.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D y");
    check(cudaMemcpyAsync(tiles_.get(), ht.data(), sizeof(TileBox) * ntiles, cudaMemcpyHostToDevice, stream_),
          "H2D tiles");
    if (geographic) {
        std::vector<TileCap> hc = make_caps(he_, kTile);
        caps_.alloc(hc.size());
        check(cudaMemcpyAsync(caps_.get(), hc.data(), sizeof(TileCap) * hc.size(), cudaMemcpyHostToDevice, stream_),
              "H2D caps");
        synchronize();
    } else {
        caps_.clear();
    }
    check(launch_build_z(n, p, x_.get(), y_.get(), z_.get(), stream_), "build_z");
    synchronize();
    hx_ = std::move(hx);
    hy_ = std::move(hy);
    hu_ = std::move(hu);
    hv_ = std::move(hv);
    recycleRanks();
    hist_.clear();
    hist_tried_ = false;
    hist_valid_ = false;
    d2c_valid_ = false;
    buildProxy();
}


void Engine::setVariables(int p, const double* x, const double* y)
{
    if (n_ == 0) throw std::logic_error("no data");
    if (p < 1 || p > kMaxP) throw std::invalid_argument("number of independent variables must be in [1, 32]");
    check(cudaSetDevice(device_), "cudaSetDevice");
    const int n = n_;
    p_ = p;
    mm_ = p * (p + 1) / 2;
    m_ = mm_ + p;
    gall_valid_ = false;
    mixed_ready_ = false;
    hx_.resize((size_t)n * p);
    hy_.resize(n);
    for (int s = 0; s < n; s++) {
        const int i = perm_[s];
        for (int k = 0; k < p; k++) hx_[(size_t)s * p + k] = x[(size_t)i + (size_t)k * n];
        hy_[s] = y[i];
    }
    x_.alloc((size_t)n * p);
    z_.alloc((size_t)n * m_);
    g_.alloc((size_t)n * m_);
    beta_.alloc((size_t)n * p);
    rvec_.alloc((size_t)n * p);
    check(cudaMemcpyAsync(x_.get(), hx_.data(), sizeof(double) * hx_.size(), cudaMemcpyHostToDevice, stream_),
          "H2D x");
    check(cudaMemcpyAsync(y_.get(), hy_.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D y");
    check(launch_build_z(n, p, x_.get(), y_.get(), z_.get(), stream_), "build_z");
    stats_.kernel_launches += 1;
    synchronize();
}

void Engine::fitDevice(double bw, bool adaptive, int kernel, bool se, double* S, double* ainv)
{
    if (n_ == 0) throw std::logic_error("no data");
    check(cudaSetDevice(device_), "cudaSetDevice");
    const int n = n_, p = p_;
    const int saved = precision_;
    precision_ = kFP64;
    struct Restore {
        int& slot;
        int value;
        double*& out;
        ~Restore()
        {
            slot = value;
            out = nullptr;
        }
    } restore{precision_, saved, ainv_out_};
    g2_.alloc((size_t)n * mm_);
    vvec_.alloc((size_t)n * p);
    bse_.alloc((size_t)n * p);
    qdiag_.alloc(n);
    computeThresholds(bw, adaptive);
    contract(z_.get(), m_, g_.get(), m_, bw, adaptive, kernel, false, 1);
    if (se)
        contract(z_.get(), mm_, g2_.get(), mm_, bw, adaptive, kernel, false, 2);
    else  // the solve still forms the (unused) SE terms from G2
        check(cudaMemsetAsync(g2_.get(), 0, sizeof(double) * g2_.size(), stream_), "memset G2");
    ainv_out_ = ainv;
    double s[4];
    solve(kSolveFit, bw, adaptive, kernel, s);
    if (s[3] > 0.0) throw NotSPDError("inv_sympd(): matrix is singular or not positive definite");
    if (S) {
        check(cudaMemsetAsync(S, 0, sizeof(double) * (size_t)n * n, stream_), "memset S");
        check(launch_tile_far_thr(n, kTile, geographic_, thrPtr(adaptive), bw, tile_thr16_.get(), stream_),
              "tile thr");
        check(launch_hat_pass(points(), geographic_, tb16_.get(), tile_thr16_.get(), x_.get(), p, vvec_.get(),
                              thrPtr(adaptive), bw, kernel, true, qdiag_.get(), S, -1, nullptr, stream_),
              "hat pass");
        stats_.kernel_launches += 2;
    }
}

void Engine::hatAll(double bw, bool adaptive, int kernel, const double* ainv, double* S0, double* SA)
{
    check(cudaSetDevice(device_), "cudaSetDevice");
    computeThresholds(bw, adaptive);
    check(launch_mgwr_hat_all(points(), geographic_, x_.get(), p_, ainv, thrPtr(adaptive), bw, kernel, S0, SA,
                              num_sms_, stream_),
          "hat all");
    stats_.kernel_launches += 1;
}

void Engine::hatUpdate(double bw, bool adaptive, int kernel, const double* T, double* SA)
{
    if (p_ != 1) throw std::logic_error("hatUpdate needs the one-variable problem");
    check(cudaSetDevice(device_), "cudaSetDevice");
    const int saved = precision_;
    precision_ = kFP64;
    struct Restore {
        int& slot;
        int value;
        ~Restore() { slot = value; }
    } restore{precision_, saved};
    computeThresholds(bw, adaptive);
    check(launch_mgwr_hat_update(points(), geographic_, tb16_.get(), x_.get(), vvec_.get(), thrPtr(adaptive), bw,
                                 kernel, T, SA, stream_),
          "hat update");
    stats_.kernel_launches += 1;
}

void Engine::copyOut(const double* dev, int cols, std::vector<double>& out)
{
    const int n = n_;
    std::vector<double> h((size_t)n * cols);
    check(cudaMemcpyAsync(h.data(), dev, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream_), "D2H");
    synchronize();
    out.assign((size_t)n * cols, 0.0);
    for (int s = 0; s < n; s++)
        for (int k = 0; k < cols; k++) out[(size_t)perm_[s] + (size_t)k * n] = h[(size_t)s * cols + k];
}

void Engine::betas(std::vector<double>& out) { copyOut(beta_.get(), p_, out); }
void Engine::betasSE(std::vector<double>& out) { copyOut(bse_.get(), p_, out); }

// FP32 proxy coordinates and 32-point tile bounds shared by the select and the
// mixed path.
void Engine::buildProxy()
{
    const int n = n_, p = p_;
    ntiles32_ = (n + 31) / 32;
    boxes32_.alloc(ntiles32_);
    std::vector<TileBox> bx(ntiles32_);
    for (int t = 0; t < ntiles32_; t++) {
        TileBox b{hu_[t * 32], hu_[t * 32], hv_[t * 32], hv_[t * 32]};
        for (int s = t * 32; s < std::min(n, (t + 1) * 32); s++) {
            b.ulo = std::min(b.ulo, hu_[s]);
            b.uhi = std::max(b.uhi, hu_[s]);
            b.vlo = std::min(b.vlo, hv_[s]);
            b.vhi = std::max(b.vhi, hv_[s]);
        }
        bx[t] = b;
    }
    // planar frame of the FP32 records and bounds: the centroid, and a slack of
    // a few ulp of the largest relative coordinate
    uc_ = vc_ = 0.0;
    double maxabs = 0.0;
    if (!geographic_) {
        for (int s = 0; s < n; s++) {
            uc_ += hu_[s];
            vc_ += hv_[s];
        }
        uc_ /= n;
        vc_ /= n;
        for (int s = 0; s < n; s++) maxabs = std::max(maxabs, std::max(std::fabs(hu_[s] - uc_), std::fabs(hv_[s] - vc_)));
    }
    slack_ = std::ldexp(maxabs, -20);
    std::vector<float4> pts = point_records(hu_, hv_, geographic_, uc_, vc_, he_);
    if (geographic_) {
        std::vector<TileCap> c32 = make_caps(he_, 32);
        caps32_.alloc(c32.size());
        check(cudaMemcpyAsync(caps32_.get(), c32.data(), sizeof(TileCap) * c32.size(), cudaMemcpyHostToDevice,
                              stream_),
              "H2D caps32");
        synchronize();
    } else {
        caps32_.clear();
    }
    rvec_.alloc((size_t)n * p);
    pts32_.alloc(pts.size());
    check(cudaMemcpyAsync(pts32_.get(), pts.data(), sizeof(float4) * pts.size(), cudaMemcpyHostToDevice, stream_),
          "H2D pts32");
    check(cudaMemcpyAsync(boxes32_.get(), bx.data(), sizeof(TileBox) * bx.size(), cudaMemcpyHostToDevice, stream_),
          "H2D boxes");
    std::vector<float4> tb = tile_bounds(hu_, hv_, geographic_, 32, uc_, vc_, slack_, he_);
    std::vector<float4> t16 = tile_bounds(hu_, hv_, geographic_, 16, uc_, vc_, slack_, he_);
    std::vector<float4> t1024 = tile_bounds(hu_, hv_, geographic_, 1024, uc_, vc_, slack_, he_);
    stb_.alloc(t1024.size());
    check(cudaMemcpyAsync(stb_.get(), t1024.data(), sizeof(float4) * t1024.size(), cudaMemcpyHostToDevice, stream_),
          "H2D super-tile bounds");
    // proxy error bands of the exact select.  The FP32 great-circle proxy is within
    // 5.3e-7 relative of the reference's distance wherever it is trusted (d < 15,000 km;
    // measured over near, regional and global pairs), 1e-10 km absolute for nearly
    // coincident points: 2^-16 (1.5e-5) and 1e-6 km leave a margin of 25x over it.
    // Every point inside the band is evaluated with the correctly rounded formula.
    if (!geographic_) {
        sel_eps_ = std::ldexp(1.0, -18);
        sel_delta_ = std::ldexp(dhi_, -36);
    } else {
        sel_eps_ = std::ldexp(1.0, -16);
        sel_delta_ = 1e-6;
    }
    tbsel_.alloc(tb.size());
    check(cudaMemcpyAsync(tbsel_.get(), tb.data(), sizeof(float4) * tb.size(), cudaMemcpyHostToDevice, stream_),
          "H2D tile bounds");
    tb16_.alloc(t16.size());
    check(cudaMemcpyAsync(tb16_.get(), t16.data(), sizeof(float4) * t16.size(), cudaMemcpyHostToDevice, stream_),
          "H2D tile bounds");
    tile_thr16_.alloc(t16.size());
    sel_err_.alloc(1);
    check(cudaMemsetAsync(sel_err_.get(), 0, sizeof(int), stream_), "memset");
    synchronize();
}

// Mixed-precision operands: X and y centred (when a constant column is the
// intercept) and scaled, Z~ split into TF32 hi/lo swizzled tile images, FP32
// hi/lo coordinates, 32-point tile boxes.
void Engine::ensureMixed()
{
    if (mixed_ready_) return;
    const int n = n_, p = p_;
    if (m_ > 256) throw std::invalid_argument("mixed precision supports at most 21 columns of X");
    // column statistics in two row-major passes over fixed blocks of rows (the
    // block partials are summed in block order, so the result does not depend
    // on the host's thread count)
    const size_t B = 4096, nblk = ((size_t)n + B - 1) / B;
    std::vector<double> bsum(nblk * p, 0.0), bss(nblk * p, 0.0);
    std::vector<char> bconst(nblk * p, 1);
    parallel_for(nblk, 1, [&](size_t b0, size_t b1) {
        for (size_t b = b0; b < b1; b++) {
            double* sum = &bsum[b * p];
            char* cst = &bconst[b * p];
            for (size_t s = b * B; s < std::min((size_t)n, (b + 1) * B); s++)
                for (int k = 0; k < p; k++) {
                    const double v = hx_[s * p + k];
                    sum[k] += v;
                    if (v != hx_[k]) cst[k] = 0;
                }
        }
    });
    intercept_col_ = -1;
    for (int k = 0; k < p && intercept_col_ < 0; k++) {
        bool constant = hx_[k] != 0.0;
        for (size_t b = 0; b < nblk && constant; b++) constant = bconst[b * p + k] != 0;
        if (constant) intercept_col_ = k;
    }
    mu_.assign(p, 0.0);
    sc_.assign(p, 1.0);
    if (intercept_col_ >= 0)
        for (int k = 0; k < p; k++) {
            double t = 0.0;
            for (size_t b = 0; b < nblk; b++) t += bsum[b * p + k];
            mu_[k] = k == intercept_col_ ? 0.0 : t / n;
        }
    parallel_for(nblk, 1, [&](size_t b0, size_t b1) {
        for (size_t b = b0; b < b1; b++) {
            double* ss = &bss[b * p];
            for (size_t s = b * B; s < std::min((size_t)n, (b + 1) * B); s++)
                for (int k = 0; k < p; k++) {
                    const double d = hx_[s * p + k] - mu_[k];
                    ss[k] += d * d;
                }
        }
    });
    for (int k = 0; k < p; k++) {
        if (k == intercept_col_) {
            sc_[k] = hx_[k];
            continue;
        }
        double ss = 0.0;
        for (size_t b = 0; b < nblk; b++) ss += bss[b * p + k];
        const double sd = std::sqrt(ss / n);
        sc_[k] = (sd > 0.0 && std::isfinite(sd)) ? sd : 1.0;
    }
    mu_y_ = 0.0;
    if (intercept_col_ >= 0) {
        for (int s = 0; s < n; s++) mu_y_ += hy_[s];
        mu_y_ /= n;
    }
    double ssy = 0.0;
    for (int s = 0; s < n; s++) ssy += (hy_[s] - mu_y_) * (hy_[s] - mu_y_);
    s_y_ = std::sqrt(ssy / n);
    if (!(s_y_ > 0.0) || !std::isfinite(s_y_)) s_y_ = 1.0;

    std::vector<double> xs((size_t)n * p), ys(n);
    parallel_for((size_t)n, 4096, [&](size_t b, size_t e) {
        for (size_t s = b; s < e; s++) {
            for (int k = 0; k < p; k++) xs[s * p + k] = (hx_[s * p + k] - mu_[k]) / sc_[k];
            ys[s] = (hy_[s] - mu_y_) / s_y_;
        }
    });
    std::vector<double> tinv(p), tvec(p, 0.0);
    for (int k = 0; k < p; k++) tinv[k] = 1.0 / sc_[k];
    if (intercept_col_ >= 0) {
        const double c = sc_[intercept_col_];
        for (int k = 0; k < p; k++) tvec[k] = (k == intercept_col_) ? 1.0 / c : -mu_[k] / (c * sc_[k]);
    }

    npad_ = (m_ + 15) / 16 * 16;  // the accumulator width: the tcgen05 N of an M = 128 MMA is a multiple of 16
    xs_.alloc((size_t)n * p);
    ys_.alloc(n);
    zs_.alloc((size_t)n * m_);
    zimg_.alloc((size_t)ntiles32_ * 2 * npad_ * 128);
    acc_.alloc((size_t)(n + 127) / 128 * 128 * npad_);  // rows in groups of 128 (the contraction's layout)
    stage_.alloc((size_t)(n + 127) / 128 * 128 * npad_);
    thr32_.alloc(n);
    err_.alloc(1);
    tinv_.alloc(p);
    tvec_.alloc(p);

    check(cudaMemcpyAsync(xs_.get(), xs.data(), sizeof(double) * xs.size(), cudaMemcpyHostToDevice, stream_),
          "H2D xs");
    check(cudaMemcpyAsync(ys_.get(), ys.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_), "H2D ys");
    check(cudaMemcpyAsync(tinv_.get(), tinv.data(), sizeof(double) * p, cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemcpyAsync(tvec_.get(), tvec.data(), sizeof(double) * p, cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemsetAsync(err_.get(), 0, sizeof(int), stream_), "memset err");
    check(launch_build_z(n, p, xs_.get(), ys_.get(), zs_.get(), stream_), "build_z");
    check(launch_build_zimg(n, m_, npad_, zs_.get(), m_, zimg_.get(), stream_), "build_zimg");
    synchronize();
    mixed_ready_ = true;
}

cudaEvent_t Engine::timerBegin()
{
    cudaEvent_t e0 = nullptr;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventRecord(e0, stream_), "event record");
    return e0;
}

void Engine::timerEnd(cudaEvent_t e0, int kind)
{
    cudaEvent_t e1 = nullptr;
    check(cudaEventCreate(&e1), "event");
    check(cudaEventRecord(e1, stream_), "event record");
    pending_.push_back(PendingTiming{e0, e1, kind});
}

EngineStats& Engine::stats()
{
    for (auto& pt : pending_) {
        float ms = 0.f;
        if (cudaEventSynchronize(pt.e1) == cudaSuccess && cudaEventElapsedTime(&ms, pt.e0, pt.e1) == cudaSuccess)
            (pt.kind == 0 ? stats_.contract_ms : pt.kind == 1 ? stats_.select_ms : stats_.d2c_fill_ms) += ms;
        cudaEventDestroy(pt.e0);
        cudaEventDestroy(pt.e1);
    }
    pending_.clear();
    if (counters_dirty_ && tile_count_.get()) {
        unsigned long long tiles = 0, pc[kTcProfSlots];
        check(cudaMemcpyAsync(&tiles, tile_count_.get(), sizeof(tiles), cudaMemcpyDeviceToHost, stream_), "D2H");
        check(cudaMemcpyAsync(pc, tc_prof_.get(), sizeof(pc), cudaMemcpyDeviceToHost, stream_), "D2H");
        check(cudaMemsetAsync(tile_count_.get(), 0, sizeof(unsigned long long), stream_), "memset tiles");
        check(cudaMemsetAsync(tc_prof_.get(), 0, sizeof(pc), stream_), "memset prof");
        synchronize();
        stats_.contract_tiles += (long long)tiles;
        for (int q = 0; q < kTcProfSlots && q < 12; q++) {
            if (q == kTcProfLoopMax || q == kTcProfTilesMax)
                stats_.contract_phase_cycles[q] = std::max(stats_.contract_phase_cycles[q], (double)pc[q]);
            else
                stats_.contract_phase_cycles[q] += (double)pc[q];
        }
        counters_dirty_ = false;
    }
    return stats_;
}

void Engine::resetStats()
{
    stats();
    stats_ = EngineStats{};
}

void Engine::contractMixed(double* G, int ldg, int mcols, double bw, bool adaptive, int kernel, bool exclude_self,
                           int wpow)
{
    if (adaptive) {
        check(launch_to_float(n_, thr_.get(), thr32_.get(), stream_), "thr32");
        stats_.kernel_launches += 1;
    }
    TcArgs a{};
    a.n = n_;
    a.mcols = mcols;
    a.npad = npad_;
    a.ntiles = ntiles32_;
    a.pts = pts32_.get();
    a.tb = tbsel_.get();
    a.zimg = zimg_.get();
    a.thr = adaptive ? thr32_.get() : nullptr;
    a.bw = (float)bw;
    a.kernel = kernel;
    a.exclude_self = exclude_self ? 1 : 0;
    a.skip = 1;
    a.flush_tiles = flush_tiles_;
    a.wait_limit = tc_wait_limit_;
    a.wpow = wpow;
    a.acc = acc_.get();
    a.stage = stage_.get();
    a.G = G;
    a.ldg = ldg;
    a.err = err_.get();
    // geographic: the pair distances come from the device's distance cache when it fits
    DeviceD2Cache& dc = device_d2c(device_);
    std::unique_lock<std::mutex> d2lock(dc.mu, std::defer_lock);
    if (geographic_ && d2c_limit_bytes_ != 0) {
        d2lock.lock();
        a.d2c = ensureDistanceCache();
        if (!a.d2c) d2lock.unlock();
    }
    cudaEvent_t e0 = stats_on_ ? timerBegin() : nullptr;
    if (stats_on_) {
        if (!tile_count_.get()) {
            tile_count_.alloc(1);
            tc_prof_.alloc(kTcProfSlots);
            check(cudaMemsetAsync(tile_count_.get(), 0, sizeof(unsigned long long), stream_), "memset tiles");
            check(cudaMemsetAsync(tc_prof_.get(), 0, sizeof(unsigned long long) * kTcProfSlots, stream_),
                  "memset prof");
        }
        a.tiles = tile_count_.get();
        a.prof = phases_on_ ? tc_prof_.get() : nullptr;
        counters_dirty_ = true;
    }
    check(launch_contract_tc(a, geographic_, stream_), "contract_tc");
    stats_.kernel_launches += 1;
    if (a.d2c) {
        check(cudaEventRecord(dc.used, stream_), "cudaEventRecord");
        d2lock.unlock();
    }
    if (stats_on_) {
        timerEnd(e0, 0);
        stats_.contract_launches += 1;
        double pairs = (double)n_ * n_;
        if (adaptive && kernel >= GW_KERNEL_BISQUARE) pairs = (double)n_ * std::max(0.0, std::min(bw, (double)n_) - 1);
        stats_.contract_flops += 2.0 * mcols * pairs;
        stats_.contract_bytes += 2.0 * npad_ * 128.0 * ntiles32_ * 2 + 8.0 * n_ * mcols + 16.0 * n_;
        if (a.d2c) stats_.contract_bytes += 4.0 * pairs;  // the cached distances of the nonzero pairs
    }
}

void Engine::tcSelftest(int N, const float* A, const float* B, float* D)
{
    check(cudaSetDevice(device_), "cudaSetDevice");
    DevBuf<float> dA, dB, dD;
    DevBuf<int> derr;
    dA.alloc(128 * 32);
    dB.alloc((size_t)N * 32);
    dD.alloc((size_t)128 * N);
    derr.alloc(1);
    check(cudaMemcpyAsync(dA.get(), A, sizeof(float) * 128 * 32, cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemcpyAsync(dB.get(), B, sizeof(float) * N * 32, cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemsetAsync(derr.get(), 0, sizeof(int), stream_), "memset");
    check(launch_tc_selftest(dA.get(), dB.get(), dD.get(), N, derr.get(), stream_), "tc selftest");
    int err = 0;
    check(cudaMemcpyAsync(D, dD.get(), sizeof(float) * 128 * N, cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(&err, derr.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "D2H");
    synchronize();
    if (err) throw CudaError("tensor-core self-test: a bounded wait timed out");
}

// Per-row order statistic of the given rank (1-based), computed once and kept
// for the dataset.  The first select also stores every row's histogram of
// proxy distances, so later ranks start from the right histogram bin.
const double* Engine::orderStatistic(unsigned rank)
{
    const bool exact = precision_ == kFP64;
    for (auto& e : ranks_)
        if (e->exact == exact && e->rank == rank) return e->v.get();
    if (ranks_.size() >= 64) recycleRanks();
    if (!hist_tried_) {
        hist_tried_ = true;
        const size_t bytes = (size_t)n_ * (4096 + 64) * sizeof(unsigned);
        bool fits;
        if (hist_limit_bytes_ >= 0) {
            fits = bytes <= (size_t)hist_limit_bytes_;
        } else {
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            fits = bytes < free_b / 4 || bytes <= hist_.capacityBytes() + hcoarse_.capacityBytes();
        }
        if (fits) {
            hist_.alloc((size_t)n_ * 4096);
            hcoarse_.alloc((size_t)n_ * 64);
        }
        hist_valid_ = false;
    }
    std::unique_ptr<RankStat> r;
    if (!rank_pool_.empty()) {
        r = std::move(rank_pool_.back());
        rank_pool_.pop_back();
    } else {
        r.reset(new RankStat);
    }
    r->rank = rank;
    r->exact = exact;
    r->v.alloc(n_);
    SelectArgs a{};
    a.n = n_;
    a.ntiles = ntiles32_;
    a.P = points();
    a.pts = pts32_.get();
    a.tb = tbsel_.get();
    a.stb = stb_.get();
    a.hist_cache = hist_.get();
    a.cache_valid = hist_valid_ ? 1 : 0;
    a.hist_coarse = hist_.get() ? hcoarse_.get() : nullptr;
    a.rank = rank;
    a.dlo = dlo_;
    a.dhi = dhi_;
    a.eps = sel_eps_;
    a.delta = sel_delta_;
    a.out = r->v.get();
    a.err = sel_err_.get();
    if (hist_.get() && !hist_valid_) {
        // geographic mixed data: the distance cache is filled first (each pair once,
        // the distance being symmetric) and the histograms are read back from it
        DeviceD2Cache& dc = device_d2c(device_);
        std::unique_lock<std::mutex> lk(dc.mu, std::defer_lock);
        const float* cache = nullptr;
        if (geographic_ && precision_ == kMixed && d2c_limit_bytes_ != 0) {
            lk.lock();
            cache = ensureDistanceCache();
            if (!cache) lk.unlock();
        }
        if (cache) {
            a.d2c = cache;
            check(launch_select_hist_cached(a, num_sms_, stream_), "select histograms");
            a.d2c = nullptr;
            check(cudaEventRecord(dc.used, stream_), "cudaEventRecord");
            lk.unlock();
        } else {
            check(launch_select_hist(a, geographic_, num_sms_, stream_), "select histograms");
        }
        stats_.kernel_launches += 1;
        hist_valid_ = true;
        a.cache_valid = 1;
    }
    // geographic mixed data whose distance cache is filled: the select reads the
    // histogram pass's proxy values from it instead of recomputing them
    DeviceD2Cache& dc = device_d2c(device_);
    std::unique_lock<std::mutex> lk(dc.mu, std::defer_lock);
    if (geographic_ && precision_ == kMixed && d2c_valid_) {
        lk.lock();
        if (dc.owner == this && d2c_valid_ && dc.ptr) a.d2c = dc.ptr;
        else lk.unlock();
    }
    check(launch_select(a, geographic_, exact, num_sms_, stream_), "select");
    stats_.kernel_launches += 1;
    if (a.d2c) {
        check(cudaEventRecord(dc.used, stream_), "cudaEventRecord");
        lk.unlock();
    }
    if (hist_.get()) hist_valid_ = true;
    ranks_.push_back(std::move(r));
    return ranks_.back()->v.get();
}

void Engine::computeThresholds(double bw, bool adaptive)
{
    if (!adaptive) return;
    if (thr_valid_ && thr_bw_ == bw && thr_prec_ == precision_) return;
    const double dn = bw / n_;
    cudaEvent_t e0 = stats_on_ ? timerBegin() : nullptr;
    if (dn < 1) {
        // d0 = vdist(int(b0) - 1), d1 = vdist(int(b0)) (BandwidthWeight.cpp:46-48)
        const double b0 = std::floor(bw), bx = bw - b0;
        const long long r0 = (long long)(int)b0;
        if (r0 < 1 || r0 >= n_) throw std::out_of_range("Mat::operator(): index out of bounds");
        const double* d0 = orderStatistic((unsigned)r0);
        const double* d1 = bx != 0.0 ? orderStatistic((unsigned)(r0 + 1)) : nullptr;
        check(launch_threshold_combine(n_, bw, d0, d1, thr_.get(), stream_), "threshold");
    stats_.kernel_launches += 1;
    } else {
        // fixbw = dn * max(dist) (BandwidthWeight.cpp:50-53)
        const double* dmax = orderStatistic((unsigned)n_);
        check(launch_threshold_combine(n_, bw, dmax, nullptr, thr_.get(), stream_), "threshold");
    stats_.kernel_launches += 1;
    }
    if (stats_on_) {
        timerEnd(e0, 1);
        stats_.select_launches += 1;
    }
    thr_valid_ = true;
    thr_bw_ = bw;
    thr_prec_ = precision_;
}

void Engine::contract(const double* Z, int mcols, double* G, int ldg, double bw, bool adaptive, int kernel,
                      bool exclude_self, int wpow)
{
    cudaEvent_t e0 = stats_on_ ? timerBegin() : nullptr;
    // the kernel takes at most 256 columns (p <= 21); wider Z (p up to 32) in column chunks
    for (int c0 = 0; c0 < mcols; c0 += 256) {
        const int w = std::min(256, mcols - c0);
        check(launch_contract64(points(), geographic_, tb16_.get(), Z + c0, m_, w, G + c0, ldg, thrPtr(adaptive), bw,
                                kernel, exclude_self, wpow, true, stream_),
              "contract64");
        stats_.kernel_launches += 1;
    }
    if (stats_on_) {
        timerEnd(e0, 0);
        stats_.contract_launches += 1;
        // useful pairs: dense kernels touch every pair; adaptive compact kernels
        // have b-1 neighbours with d < r_i per row (ties aside)
        double pairs = (double)n_ * n_;
        if (adaptive && kernel >= GW_KERNEL_BISQUARE) pairs = (double)n_ * std::max(0.0, std::min(bw, (double)n_) - 1);
        stats_.contract_flops += 2.0 * mcols * pairs;
        stats_.contract_bytes += 8.0 * ((double)n_ * m_ + (double)n_ * mcols) + 16.0 * n_;
    }
}

void Engine::solve(int mode, double bw, bool adaptive, int kernel, double out[4])
{
    SolveArgs a{};
    a.n = n_;
    a.p = p_;
    a.mode = mode;
    a.kernel = kernel;
    a.G = g_.get();
    a.ldg = m_;
    a.G2 = g2_.get();
    a.ldg2 = mm_;
    const bool mixed = precision_ == kMixed;
    a.X = mixed ? xs_.get() : x_.get();
    a.y = mixed ? ys_.get() : y_.get();
    a.thr = thrPtr(adaptive);
    a.bw = bw;
    // the criteria need no coefficients (the solve then skips the backward substitution)
    a.beta = (mode == kSolveAIC || mode == kSolveCV) ? nullptr : beta_.get();
    a.sii = sii_.get();
    a.resid = resid_.get();
    a.v = vvec_.get();
    a.bse = bse_.get();
    a.partials = partials_.get();
    a.tinv = mixed ? tinv_.get() : nullptr;
    a.tvec = (mixed && intercept_col_ >= 0) ? tvec_.get() : nullptr;
    a.tcol = mixed ? intercept_col_ : -1;
    a.rvec = rvec_.get();
    a.ainv = mode == kSolveFit ? ainv_out_ : nullptr;
    int nb = 0;
    check(launch_solve(a, &nb, stream_), "solve");
    check(launch_reduce_partials(partials_.get(), nb, sums_.get(), stream_), "reduce");
    check(cudaMemcpyAsync(host_sums_, sums_.get(), 4 * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H sums");
    if (mixed) check(cudaMemcpyAsync(host_sums_ + 4, err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(host_sums_ + 5, sel_err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "D2H");
    synchronize();
    for (int q = 0; q < 4; q++) out[q] = host_sums_[q];
    {
        int serr = 0;
        std::memcpy(&serr, host_sums_ + 5, sizeof(int));
        if (serr) throw CudaError("adaptive threshold select failed (code " + std::to_string(serr) + ")");
    }
    if (mixed) {
        int err = 0;
        std::memcpy(&err, host_sums_ + 4, sizeof(int));
        if (err) {
            // clear the flag so that the engine's next call starts clean
            check(cudaMemsetAsync(err_.get(), 0, sizeof(int), stream_), "memset err");
            synchronize();
            throw CudaError("tensor-core contraction: a bounded wait timed out");
        }
        out[1] *= s_y_ * s_y_;  // RSS / CV in the units of y
    }
}

// One refinement step of every local solve (mixed path): residual of the
// normal equations in FP64 over the contraction's weights, then beta += A~^-1 r.
void Engine::refine(double bw, bool adaptive, int kernel, double out[4])
{
    RefineArgs r{};
    r.n = n_;
    r.p = p_;
    r.ntiles = ntiles32_;
    r.kernel = kernel;
    r.skip = 1;
    r.pts = pts32_.get();
    r.tb = tbsel_.get();
    r.X = xs_.get();
    r.y = ys_.get();
    r.beta = beta_.get();
    r.thr = adaptive ? thr32_.get() : nullptr;
    r.bw = (float)bw;
    r.r = rvec_.get();
    // geographic: the contraction's distances from the device's distance cache, as the contraction read them
    DeviceD2Cache& dc = device_d2c(device_);
    std::unique_lock<std::mutex> d2lock(dc.mu, std::defer_lock);
    if (geographic_ && d2c_limit_bytes_ != 0) {
        d2lock.lock();
        r.d2c = ensureDistanceCache();
        if (!r.d2c) d2lock.unlock();
    }
    check(launch_refine_residual(r, geographic_, stream_), "refine residual");
    stats_.kernel_launches += 1;
    if (r.d2c) {
        check(cudaEventRecord(dc.used, stream_), "cudaEventRecord");
        d2lock.unlock();
    }
    solve(kSolveRefine, bw, adaptive, kernel, out);
}

double Engine::criterion(double bw, bool adaptive, int kernel, int crit)
{
    if (n_ == 0) throw std::logic_error("no data");
    check(cudaSetDevice(device_), "cudaSetDevice");
    if (precision_ == kMixed) ensureMixed();
    computeThresholds(bw, adaptive);
    if (precision_ == kMixed)
        contractMixed(g_.get(), m_, m_, bw, adaptive, kernel, crit == kCV, 1);
    else
        contract(z_.get(), m_, g_.get(), m_, bw, adaptive, kernel, crit == kCV, 1);
    double s[4];
    solve(crit == kCV ? kSolveCV : kSolveAIC, bw, adaptive, kernel, s);
    if (precision_ == kMixed && refine_search_ && crit == kAIC && s[3] == 0.0) {
        // refine beta (and so RSS); the CV criterion excludes w_ii and is not refined
        double r[4];
        for (int it = 0; it < refine_steps_; it++) refine(bw, adaptive, kernel, r);
        if (refine_steps_ > 0) s[1] = r[1];
    }
    stats_.criterion_evals++;
    if (s[3] > 0.0) return DBL_MAX;
    if (crit == kCV) return std::isfinite(s[1]) ? s[1] : DBL_MAX;
    double v = aicc((double)n_, s[1], s[0]);
    return std::isfinite(v) ? v : DBL_MAX;
}

void Engine::fit(double bw, bool adaptive, int kernel, bool storeS, FitOutput& out)
{
    if (n_ == 0) throw std::logic_error("no data");
    check(cudaSetDevice(device_), "cudaSetDevice");
    const int n = n_, p = p_;
    g2_.alloc((size_t)n * mm_);
    vvec_.alloc((size_t)n * p);
    bse_.alloc((size_t)n * p);
    qdiag_.alloc(n);
    const bool mixed = precision_ == kMixed;
    if (mixed) ensureMixed();
    computeThresholds(bw, adaptive);
    if (mixed) {
        contractMixed(g_.get(), m_, m_, bw, adaptive, kernel, false, 1);
        contractMixed(g2_.get(), mm_, mm_, bw, adaptive, kernel, false, 2);
    } else {
        contract(z_.get(), m_, g_.get(), m_, bw, adaptive, kernel, false, 1);
        contract(z_.get(), mm_, g2_.get(), mm_, bw, adaptive, kernel, false, 2);
    }
    double s[4];
    solve(kSolveFit, bw, adaptive, kernel, s);
    if (s[3] > 0.0) throw NotSPDError("inv_sympd(): matrix is singular or not positive definite");
    if (mixed) {
        double r[4];
        for (int it = 0; it < refine_steps_; it++) refine(bw, adaptive, kernel, r);
        if (refine_steps_ > 0) s[1] = r[1];
    }
    // S: n x n when stored (isStoreS, GWRBasic.h:708), else only the last
    // location's row, which is what S.row(0) holds after the reference's loop
    int last_sorted = 0;
    for (int sidx = 0; sidx < n; sidx++)
        if (perm_[sidx] == n - 1) last_sorted = sidx;
    S_.alloc(storeS ? (size_t)n * n : (size_t)n);
    check(cudaMemsetAsync(S_.get(), 0, sizeof(double) * S_.size(), stream_), "memset S");
    check(launch_tile_far_thr(n, kTile, geographic_, thrPtr(adaptive), bw, tile_thr16_.get(), stream_), "tile thr");
    stats_.kernel_launches += 2;  // tile thresholds and the hat pass
    if (mixed) {
        if (adaptive) check(launch_to_float(n_, thr_.get(), thr32_.get(), stream_), "thr32");
        check(launch_hat_mixed(n, geographic_, pts32_.get(), tb16_.get(), tile_thr16_.get(), xs_.get(), p,
                               vvec_.get(), adaptive ? thr32_.get() : nullptr, (float)bw, kernel, qdiag_.get(),
                               storeS ? S_.get() : nullptr, storeS ? -1 : last_sorted, storeS ? nullptr : S_.get(),
                               stream_),
              "hat pass");
    } else {
        check(launch_hat_pass(points(), geographic_, tb16_.get(), tile_thr16_.get(), x_.get(), p, vvec_.get(),
                              thrPtr(adaptive), bw, kernel, true, qdiag_.get(), storeS ? S_.get() : nullptr,
                              storeS ? -1 : last_sorted, storeS ? nullptr : S_.get(), stream_),
              "hat pass");
    }
    std::vector<double> hb((size_t)n * p), hse((size_t)n * p), hq(n), hsii(n), hres(n);
    check(cudaMemcpyAsync(hb.data(), beta_.get(), sizeof(double) * hb.size(), cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(hse.data(), bse_.get(), sizeof(double) * hse.size(), cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(hq.data(), qdiag_.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream_), "D2H");
    std::vector<double> hS(S_.size());
    check(cudaMemcpyAsync(hS.data(), S_.get(), sizeof(double) * hS.size(), cudaMemcpyDeviceToHost, stream_), "D2H S");
    synchronize();
    out.betas.assign((size_t)n * p, 0.0);
    out.betasSE.assign((size_t)n * p, 0.0);
    out.qdiag.assign(n, 0.0);
    if (mixed) {
        // beta_k = s_y beta~_k / s_k; the intercept absorbs the centring
        for (int sidx = 0; sidx < n; sidx++) {
            double* b = &hb[(size_t)sidx * p];
            double shift = 0.0;
            for (int k = 0; k < p; k++) {
                if (k == intercept_col_) continue;
                b[k] = s_y_ * b[k] / sc_[k];
                shift += b[k] * mu_[k];
            }
            if (intercept_col_ >= 0) {
                const int c = intercept_col_;
                b[c] = (mu_y_ + s_y_ * b[c] - shift) / sc_[c];
            }
        }
    }
    for (int sidx = 0; sidx < n; sidx++) {
        const int i = perm_[sidx];
        for (int k = 0; k < p; k++) {
            out.betas[(size_t)i + (size_t)k * n] = hb[(size_t)sidx * p + k];
            out.betasSE[(size_t)i + (size_t)k * n] = hse[(size_t)sidx * p + k];
        }
        out.qdiag[i] = hq[sidx];
    }
    if (storeS) {
        out.sRows = n;
        out.S.assign((size_t)n * n, 0.0);
        for (int a = 0; a < n; a++)
            for (int b = 0; b < n; b++) out.S[(size_t)perm_[a] + (size_t)perm_[b] * n] = hS[(size_t)a * n + b];
    } else {
        out.sRows = 1;
        out.S.assign(n, 0.0);
        for (int b = 0; b < n; b++) out.S[perm_[b]] = hS[b];
    }
    out.shat[0] = s[0];
    out.shat[1] = s[2];
    out.rss = s[1];
}

double Engine::golden(bool adaptive, int kernel, int crit, double lower, double upper,
                      std::map<double, double>& record)
{
    double xopt = 0.0;
    golden_section(
        lower, upper, adaptive, [&](double b) { return criterion(b, adaptive, kernel, crit); }, [] { return true; },
        xopt, record);
    return xopt;
}

size_t Engine::estimateBytes(int n, int p, bool geographic, bool mixed, bool adaptive, long long hist_limit)
{
    const double N = n, P = p;
    const double m = P * (P + 1) / 2 + P, mm = P * (P + 1) / 2;
    const double npad = std::ceil(m / 16) * 16;
    const double t16 = std::ceil(N / 16), t32 = std::ceil(N / 32);
    const double g = geographic ? 1.0 : 0.0;
    double b = 8 * N * (2 + 5 * g);                                  // u, v, uR, vR, unit vectors
    b += 8 * N * (P + 1 + 2 * m + 3 + P + 2 + P);                    // x, y, z, g, thr, sel0/1, beta, sii, resid, rvec
    b += 8 * 16384 + 64;                                              // partials, sums
    b += 32 * t16 * (1 + g) + 32 * t32 * (1 + g);                     // tile boxes and caps (16 and 32 points)
    b += 16 * t32 * 32 * (1 + g) + 16 * t32 + 20 * t16;               // point records, tile bounds, tile thresholds
    b += 8 * N * kMaxP + 8 * (kMaxP * (kMaxP + 3) / 2 + kMaxP);       // variable-selection scratch
    const double n128 = std::ceil(N / 128) * 128;                    // rows of the contraction's sums
    if (mixed) b += 8 * N * (P + 1 + m) + t32 * 2 * npad * 128 + 12 * n128 * npad + 4 * N;
    b += 8 * N * (mm + 2 * P + 2);                                    // fit: G2, v, betasSE, qDiag, S row
    if (adaptive) {
        const double h = 4.0 * (4096 + 64) * N;  // histograms and their segment counts
        if (hist_limit < 0 || h <= (double)hist_limit) b += h;
        b += 64 * 8 * N;                                              // cached order statistics
    }
    return (size_t)(b * 1.05) + (16u << 20);
}

size_t Engine::bytesHeld() const
{
    size_t b = u_.capacityBytes() + v_.capacityBytes() + uR_.capacityBytes() + vR_.capacityBytes() + e_.capacityBytes() +
               x_.capacityBytes() + y_.capacityBytes() + z_.capacityBytes() + g_.capacityBytes() +
               thr_.capacityBytes() + sel0_.capacityBytes() + sel1_.capacityBytes() + beta_.capacityBytes() +
               sii_.capacityBytes() + resid_.capacityBytes() + partials_.capacityBytes() + sums_.capacityBytes() +
               tiles_.capacityBytes() + caps_.capacityBytes() + boxes32_.capacityBytes() + caps32_.capacityBytes() +
               rvec_.capacityBytes() + pts32_.capacityBytes() + tbsel_.capacityBytes() + tb16_.capacityBytes() +
               tile_thr16_.capacityBytes() + xs_.capacityBytes() + ys_.capacityBytes() + zs_.capacityBytes() +
               zimg_.capacityBytes() + acc_.capacityBytes() + stage_.capacityBytes() + thr32_.capacityBytes() + g2_.capacityBytes() +
               vvec_.capacityBytes() + bse_.capacityBytes() + qdiag_.capacityBytes() + S_.capacityBytes() +
               hist_.capacityBytes() + hcoarse_.capacityBytes() + xsub_.capacityBytes() + gsub_.capacityBytes() + stb_.capacityBytes();
    for (auto& r : ranks_) b += r->v.capacityBytes();
    for (auto& r : rank_pool_) b += r->v.capacityBytes();
    return b;
}

void Engine::predict(int nr, const double* locations, double bw, bool adaptive, int kernel,
                     std::vector<double>& betas)
{
    if (n_ == 0) throw std::logic_error("no data");
    if (nr < 1) throw std::invalid_argument("no prediction locations");
    check(cudaSetDevice(device_), "cudaSetDevice");
    const int p = p_;
    // prediction points in Hilbert order (for compact focus blocks)
    double umin = locations[0], umax = umin, vmin = locations[nr], vmax = vmin;
    for (int i = 0; i < nr; i++) {
        umin = std::min(umin, locations[i]);
        umax = std::max(umax, locations[i]);
        vmin = std::min(vmin, locations[nr + i]);
        vmax = std::max(vmax, locations[nr + i]);
    }
    const double su = umax > umin ? 2147483647.0 / (umax - umin) : 0.0;
    const double sv = vmax > vmin ? 2147483647.0 / (vmax - vmin) : 0.0;
    std::vector<std::pair<uint64_t, int>> keyed(nr);
    for (int i = 0; i < nr; i++) {
        const double fu = (locations[i] - umin) * su, fv = (locations[nr + i] - vmin) * sv;
        const uint32_t qu = std::isfinite(fu) ? (uint32_t)std::min(std::max(fu, 0.0), 2147483647.0) : 0u;
        const uint32_t qv = std::isfinite(fv) ? (uint32_t)std::min(std::max(fv, 0.0), 2147483647.0) : 0u;
        keyed[i] = {hilbert_index(qu, qv), i};
    }
    std::sort(keyed.begin(), keyed.end());
    std::vector<double> fu(nr), fv(nr), fuR, fvR;
    const double DE2RA = M_PI / 180;
    for (int s = 0; s < nr; s++) {
        fu[s] = locations[keyed[s].second];
        fv[s] = locations[nr + keyed[s].second];
    }
    if (geographic_) {
        fuR.resize(nr);
        fvR.resize(nr);
        for (int s = 0; s < nr; s++) {
            fuR[s] = fu[s] * DE2RA;
            fvR[s] = fv[s] * DE2RA;
        }
    }
    // the focus bounds share the data's planar frame; widen the slack to cover both
    double slack = slack_;
    if (!geographic_) {
        double maxabs = 0.0;
        for (int s = 0; s < nr; s++) maxabs = std::max(maxabs, std::max(std::fabs(fu[s] - uc_), std::fabs(fv[s] - vc_)));
        slack = std::max(slack, std::ldexp(maxabs, -20));
    }
    const std::vector<double> fe = geographic_ ? unit_vectors(fuR, fvR) : std::vector<double>();
    std::vector<float4> fpts = point_records(fu, fv, geographic_, uc_, vc_, fe);
    std::vector<float4> ftb = tile_bounds(fu, fv, geographic_, kTile, uc_, vc_, slack, fe);
    pf_u_.alloc(nr);
    pf_v_.alloc(nr);
    check(cudaMemcpyAsync(pf_u_.get(), fu.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, stream_), "H2D");
    check(cudaMemcpyAsync(pf_v_.get(), fv.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, stream_), "H2D");
    if (geographic_) {
        pf_uR_.alloc(nr);
        pf_vR_.alloc(nr);
        check(cudaMemcpyAsync(pf_uR_.get(), fuR.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, stream_), "H2D");
        check(cudaMemcpyAsync(pf_vR_.get(), fvR.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, stream_), "H2D");
        pf_e_.alloc(fe.size());
        check(cudaMemcpyAsync(pf_e_.get(), fe.data(), sizeof(double) * fe.size(), cudaMemcpyHostToDevice, stream_),
              "H2D unit vectors");
        synchronize();
    }
    pf_pts_.alloc(fpts.size());
    check(cudaMemcpyAsync(pf_pts_.get(), fpts.data(), sizeof(float4) * fpts.size(), cudaMemcpyHostToDevice, stream_),
          "H2D");
    pf_tb16_.alloc(ftb.size());
    check(cudaMemcpyAsync(pf_tb16_.get(), ftb.data(), sizeof(float4) * ftb.size(), cudaMemcpyHostToDevice, stream_),
          "H2D");
    DevPoints F;
    F.n = nr;
    F.u = pf_u_.get();
    F.v = pf_v_.get();
    F.uR = geographic_ ? pf_uR_.get() : nullptr;
    F.vR = geographic_ ? pf_vR_.get() : nullptr;
    F.e = geographic_ ? pf_e_.get() : nullptr;

    // thresholds: fixbw of BandwidthWeight.cpp:40-53 over each location's distances to the data
    const double* thr = nullptr;
    if (adaptive) {
        pf_thr_.alloc(nr);
        pf_d0_.alloc(nr);
        auto select = [&](unsigned rank, double* out) {
            SelectArgs a{};
            a.n = n_;
            a.ntiles = ntiles32_;
            a.P = points();
            a.pts = pts32_.get();
            a.tb = tbsel_.get();
            a.stb = stb_.get();
            a.hist_cache = nullptr;
            a.cache_valid = 0;
            a.rank = rank;
            a.dlo = dlo_;
            a.dhi = dhi_;
            a.eps = sel_eps_;
            a.delta = sel_delta_;
            a.out = out;
            a.err = sel_err_.get();
            a.F = F;
            a.fpts = pf_pts_.get();
            check(launch_select(a, geographic_, true, num_sms_, stream_), "predict select");
            stats_.kernel_launches += 1;
        };
        const double dn = bw / n_;
        if (dn < 1) {
            const double b0 = std::floor(bw), bx = bw - b0;
            const long long r0 = (long long)(int)b0;
            if (r0 < 1 || r0 >= n_) throw std::out_of_range("Mat::operator(): index out of bounds");
            select((unsigned)r0, pf_d0_.get());
            const double* d1 = nullptr;
            if (bx != 0.0) {
                pf_d1_.alloc(nr);
                select((unsigned)(r0 + 1), pf_d1_.get());
                d1 = pf_d1_.get();
            }
            check(launch_threshold_combine_rows(nr, n_, bw, pf_d0_.get(), d1, pf_thr_.get(), stream_), "threshold");
        } else {
            select((unsigned)n_, pf_d0_.get());
            check(launch_threshold_combine_rows(nr, n_, bw, pf_d0_.get(), nullptr, pf_thr_.get(), stream_),
                  "threshold");
        }
        stats_.kernel_launches += 1;
        thr = pf_thr_.get();
    }
    // X^T W_i X, X^T W_i y at every location, then beta_i = (X^T W_i X)^-1 X^T W_i y
    pf_g_.alloc((size_t)nr * m_);
    for (int c0 = 0; c0 < m_; c0 += 256) {  // at most 256 columns a launch
        check(launch_contract64_focus(points(), tb16_.get(), F, pf_tb16_.get(), geographic_, z_.get() + c0, m_,
                                      std::min(256, m_ - c0), pf_g_.get() + c0, m_, thr, bw, kernel, false, 1, true,
                                      stream_),
              "predict contraction");
        stats_.kernel_launches += 1;
    }
    pf_beta_.alloc((size_t)nr * p);
    SolveArgs a{};
    a.n = nr;
    a.p = p;
    a.mode = kSolvePredict;
    a.kernel = kernel;
    a.G = pf_g_.get();
    a.ldg = m_;
    a.thr = thr;
    a.bw = bw;
    a.beta = pf_beta_.get();
    a.partials = partials_.get();
    a.tcol = -1;
    int nb = 0;
    check(launch_solve(a, &nb, stream_), "predict solve");
    check(launch_reduce_partials(partials_.get(), nb, sums_.get(), stream_), "reduce");
    stats_.kernel_launches += 3;
    std::vector<double> hb((size_t)nr * p);
    check(cudaMemcpyAsync(hb.data(), pf_beta_.get(), sizeof(double) * hb.size(), cudaMemcpyDeviceToHost, stream_),
          "D2H");
    check(cudaMemcpyAsync(host_sums_, sums_.get(), 4 * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(host_sums_ + 5, sel_err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "D2H");
    synchronize();
    int serr = 0;
    std::memcpy(&serr, host_sums_ + 5, sizeof(int));
    if (serr) throw CudaError("adaptive threshold select failed (code " + std::to_string(serr) + ")");
    if (host_sums_[3] > 0.0) throw NotSPDError("inv_sympd(): matrix is singular or not positive definite");
    betas.assign((size_t)nr * p, 0.0);
    for (int s = 0; s < nr; s++) {
        const int i = keyed[s].second;
        for (int k = 0; k < p; k++) betas[(size_t)i + (size_t)k * nr] = hb[(size_t)s * p + k];
    }
}

void Engine::releaseDistanceCache()
{
    DeviceD2Cache& c = device_d2c(device_);
    std::lock_guard<std::mutex> lk(c.mu);
    d2c_valid_ = false;
    if (c.owner != this) return;
    check(cudaSetDevice(device_), "cudaSetDevice");
    free_d2c(c);
}

bool Engine::distanceCacheActive() const
{
    DeviceD2Cache& c = device_d2c(device_);
    std::lock_guard<std::mutex> lk(c.mu);
    return c.owner == this && d2c_valid_;
}

// The device's distance cache holding this dataset, filled now if needed, or
// null when the cache does not apply or does not fit.  The caller holds the
// cache's lock and records its `used` event after the launch that reads it.
const float* Engine::ensureDistanceCache()
{
    DeviceD2Cache& c = g_d2c[device_];
    if (c.owner == this && d2c_valid_ && c.ptr) return c.ptr;
    float* d2c = acquireDistanceCache();
    if (!d2c) return nullptr;
    cudaEvent_t e0 = stats_on_ ? timerBegin() : nullptr;
    fill_scratch_.alloc((size_t)(n_ + 127) / 128 + 2);
    check(launch_fill_d2_sym(n_, pts32_.get(), d2c, fill_scratch_.get(), num_sms_, stream_), "fill distance cache");
    stats_.kernel_launches += 2;
    if (stats_on_) {
        timerEnd(e0, 2);
        stats_.d2c_fills += 1;
    }
    d2c_valid_ = true;
    return d2c;
}

// The device's distance cache, owned by this engine and large enough for its
// dataset (contents not yet this dataset's: the caller fills it), or null.
// The caller holds the cache's lock.
float* Engine::acquireDistanceCache()
{
    if (!geographic_ || precision_ != kMixed || d2c_limit_bytes_ == 0 || n_ < 1) return nullptr;
    DeviceD2Cache& c = g_d2c[device_];
    d2c_valid_ = false;
    const size_t need = d2_cache_bytes(n_);
    if (d2c_limit_bytes_ > 0 && need > (size_t)d2c_limit_bytes_) return nullptr;
    if (c.bytes < need) {
        if (c.ptr) free_d2c(c);
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        const size_t reserve = std::max((size_t)16 << 30, total_b / 8);
        if (need + reserve > free_b) return nullptr;
        if (cudaMalloc(&c.ptr, need) != cudaSuccess) {
            cudaGetLastError();  // too little memory after all: run without the cache
            c.ptr = nullptr;
            return nullptr;
        }
        c.bytes = need;
        c.owner = nullptr;
    }
    if (!c.used) check(cudaEventCreateWithFlags(&c.used, cudaEventDisableTiming), "cudaEventCreate");
    // the previous owner's launches that read the buffer come first
    if (c.owner && c.owner != this) check(cudaStreamWaitEvent(stream_, c.used, 0), "cudaStreamWaitEvent");
    c.owner = this;
    return c.ptr;
}

void Engine::clearCaches()
{
    d2c_valid_ = false;
    recycleRanks();
    hist_valid_ = false;
    thr_valid_ = false;
    gall_valid_ = false;
}

void Engine::recordEvent(int slot)
{
    if (slot < 0 || slot >= 8) throw std::invalid_argument("event slot out of range");
    check(cudaSetDevice(device_), "cudaSetDevice");
    if (!events_[slot]) check(cudaEventCreate(&events_[slot]), "cudaEventCreate");
    check(cudaEventRecord(events_[slot], stream_), "cudaEventRecord");
}

float Engine::elapsedMs(int a, int b)
{
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !events_[a] || !events_[b])
        throw std::invalid_argument("event slot not recorded");
    check(cudaEventSynchronize(events_[b]), "cudaEventSynchronize");
    float ms = 0.f;
    check(cudaEventElapsedTime(&ms, events_[a], events_[b]), "cudaEventElapsedTime");
    return ms;
}

double Engine::globalCriterion(const std::vector<int>& cols)
{
    if (n_ == 0) throw std::logic_error("no data");
    const int q = (int)cols.size();
    if (q < 1 || q > kMaxP) throw std::invalid_argument("column subset size out of range");
    check(cudaSetDevice(device_), "cudaSetDevice");
    if (!gall_valid_) {
        const int nb = 256;
        gall_.alloc(m_);
        gall_part_.alloc((size_t)nb * m_);
        check(launch_column_sums(n_, m_, z_.get(), gall_part_.get(), nb, gall_.get(), stream_), "column sums");
        gall_valid_ = true;
    }
    ColumnSet cs{};
    cs.count = q;
    for (int a = 0; a < q; a++) {
        if (cols[a] < 0 || cols[a] >= p_) throw std::invalid_argument("column index out of range");
        cs.cols[a] = cols[a];
    }
    xsub_.alloc((size_t)n_ * kMaxP);
    gsub_.alloc((size_t)kMaxP * (kMaxP + 3) / 2 + kMaxP);
    check(launch_gather_subset(n_, p_, cs, x_.get(), gall_.get(), xsub_.get(), gsub_.get(), stream_), "gather");
    SolveArgs a{};
    a.n = n_;
    a.p = q;
    a.mode = kSolveAIC;
    a.kernel = GW_KERNEL_GAUSSIAN;  // w_ii = exp(0) = 1
    a.G = gsub_.get();
    a.ldg = 0;                      // every location solves the same X^T X
    a.X = xsub_.get();
    a.y = y_.get();
    a.thr = nullptr;
    a.bw = 1.0;
    a.beta = nullptr;
    a.sii = sii_.get();
    a.resid = resid_.get();
    a.partials = partials_.get();
    int nb = 0;
    check(launch_solve(a, &nb, stream_), "solve");
    check(launch_reduce_partials(partials_.get(), nb, sums_.get(), stream_), "reduce");
    check(cudaMemcpyAsync(host_sums_, sums_.get(), 4 * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H sums");
    synchronize();
    if (host_sums_[3] > 0.0) return DBL_MAX;
    double v = aicc((double)n_, host_sums_[1], host_sums_[0]);
    return std::isfinite(v) ? v : DBL_MAX;
}

double Engine::maxDistance()
{
    check(cudaSetDevice(device_), "cudaSetDevice");
    check(cudaMemsetAsync(key_.get(), 0, 2 * sizeof(unsigned long long), stream_), "memset");
    if (geographic_) rowmax_.alloc(n_);
    check(launch_max_distance(points(), geographic_, key_.get(), rowmax_.get(), num_sms_, stream_), "maxdist");
    unsigned long long k = 0;
    check(cudaMemcpyAsync(&k, key_.get() + (geographic_ ? 1 : 0), sizeof(k), cudaMemcpyDeviceToHost, stream_),
          "D2H");
    synchronize();
    uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

void Engine::thresholds(double bw, bool adaptive, std::vector<double>& out)
{
    check(cudaSetDevice(device_), "cudaSetDevice");
    out.assign(n_, bw);
    if (!adaptive) return;
    computeThresholds(bw, adaptive);
    std::vector<double> h(n_);
    int serr = 0;
    check(cudaMemcpyAsync(h.data(), thr_.get(), sizeof(double) * n_, cudaMemcpyDeviceToHost, stream_), "D2H");
    check(cudaMemcpyAsync(&serr, sel_err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "D2H");
    synchronize();
    if (serr) throw CudaError("adaptive threshold select failed (code " + std::to_string(serr) + ")");
    for (int s = 0; s < n_; s++) out[perm_[s]] = h[s];
}

}  // namespace gwgpu
