// engine.h -- the device-resident GWR engine behind the C ABI and the
// gwm::GWRBasic facade.  One engine owns one dataset on one GPU and one
// stream; it is not re-entrant (serialize calls per engine).
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gw_common.cuh"

namespace gwgpu {

enum Precision { kFP64 = 0, kMixed = 1 };
enum Criterion { kAIC = 0, kCV = 1 };

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

// A local X^T W X that is not symmetric positive definite; mirrors the
// std::runtime_error of inv_sympd / "Cuda failed to get the inverse of matrix".
struct NotSPDError : std::runtime_error {
    explicit NotSPDError(const std::string& s) : std::runtime_error(s) {}
};

void check(cudaError_t e, const char* what);

template <class T>
class DevBuf {
public:
    DevBuf() = default;
    ~DevBuf() { release(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    // Grow-only: a smaller request keeps the allocation, so an engine that is
    // reused for datasets of different sizes stops calling cudaMalloc and
    // cudaFree (both synchronise the device) once it has seen the largest.
    void alloc(size_t count)
    {
        if (count <= cap_ && ptr_) {
            count_ = count;
            return;
        }
        release();
        if (count) check(cudaMalloc(&ptr_, count * sizeof(T)), "cudaMalloc");
        count_ = cap_ = count;
    }
    // Empty (get() returns null) without freeing the allocation.
    void clear() { count_ = 0; }
    void release()
    {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        count_ = cap_ = 0;
    }
    T* get() const { return count_ ? ptr_ : nullptr; }
    size_t size() const { return count_; }
    size_t capacityBytes() const { return cap_ * sizeof(T); }

private:
    T* ptr_ = nullptr;
    size_t count_ = 0, cap_ = 0;
};

// Timing of the contraction launches, filled when stats are enabled.
struct EngineStats {
    int contract_launches = 0;
    double contract_ms = 0.0;      // sum of event-timed contraction launches
    double contract_flops = 0.0;   // algorithmic 2 * m * P, P = nonzero weight pairs
    double contract_bytes = 0.0;   // algorithmic Z + G + coordinate bytes
    long long contract_tiles = 0;  // 128 x 32 weight tiles the mixed contraction processed
    double contract_phase_cycles[12] = {};  // mixed contraction: clock64 cycles per TcProf phase
    int select_launches = 0;
    double select_ms = 0.0;
    double solve_ms = 0.0;
    int criterion_evals = 0;
    long long kernel_launches = 0;  // kernels launched by the engine (always counted)
    int d2c_fills = 0;              // distance cache fills
    double d2c_fill_ms = 0.0;       // their event-timed duration
};

struct FitOutput {
    std::vector<double> betas;     // n x p column-major (original order)
    std::vector<double> betasSE;   // n x p, before the sigma scaling of GWRBasic::fit
    std::vector<double> qdiag;     // n
    std::vector<double> S;         // sRows x n column-major
    int sRows = 0;
    double shat[2] = {0.0, 0.0};
    double rss = 0.0;
};

class Engine {
public:
    explicit Engine(int device);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // Copies X (n x p column-major), y and coords (n x 2 column-major) to the
    // device in Hilbert order.
    void setData(int n, int p, const double* x, const double* y, const double* coords, bool geographic);
    // Replaces X (n x p column-major) and y, keeping the coordinates, their
    // order and every distance cache (thresholds, order statistics,
    // histograms): the per-variable problems of GWRMultiscale share one geometry.
    void setVariables(int p, const double* x, const double* y);
    // FP64 fit that leaves its results on the device: beta, with se the
    // diagonal of C C^T (C = A_i^-1 X^T W_i, GWRMultiscale.cpp:216-224), and,
    // when the pointers are set, S (n x n row-major, sorted order) and the
    // local inverses A_i^-1 (n x p x p).  Throws NotSPDError.
    void fitDevice(double bw, bool adaptive, int kernel, bool se, double* S, double* ainv);
    // SA_k and S0 of the initial all-variable fit from fitDevice's inverses.
    void hatAll(double bw, bool adaptive, int kernel, const double* ainv, double* S0, double* SA);
    // SA = S (T + I) with S the hat matrix of the last one-variable fitDevice
    // at this bandwidth (a compact kernel), over neighbouring tiles only.
    void hatUpdate(double bw, bool adaptive, int kernel, const double* T, double* SA);
    // beta / betasSE of the last fitDevice, n x p column-major in the original order.
    void betas(std::vector<double>& out);
    void betasSE(std::vector<double>& out);
    void setPrecision(int precision) { precision_ = precision; }
    // Tiles per FP32 accumulation chunk of the tensor-core contraction (>= 2).
    void setFlushTiles(int tiles) { flush_tiles_ = tiles; }
    // Polls of the tensor-core contraction's pipeline waits before they time out
    // (0: the default, about two seconds); small values exercise the timeout path.
    void setTcWaitLimit(unsigned polls) { tc_wait_limit_ = polls; }
    int flushTiles() const { return flush_tiles_; }
    // Refinement steps of the mixed final fit (and of each search criterion when refine_search).
    void setRefinement(int steps, bool refine_search)
    {
        refine_steps_ = steps;
        refine_search_ = refine_search;
    }
    int precision() const { return precision_; }
    // Largest histogram cache (bytes) the adaptive select may allocate; -1
    // lets it take up to a quarter of the free device memory.
    void setHistLimit(long long bytes) { hist_limit_bytes_ = bytes; }
    // Upper bound of the device memory an engine holds after setData plus a
    // search and a fit of a dataset of this shape (the allocations below).
    static size_t estimateBytes(int n, int p, bool geographic, bool mixed, bool adaptive, long long hist_limit);
    // Device memory currently held (capacity of every buffer).
    size_t bytesHeld() const;

    int n() const { return n_; }
    int p() const { return p_; }

    // bandwidthSizeCriterion{AIC,CV}: DBL_MAX when a local system is not SPD
    // or the value is not finite (GWRBasic.cpp:440-535).  shat receives
    // (trS, trStS-unused) for AIC.
    double criterion(double bw, bool adaptive, int kernel, int crit);
    // fitOmp outputs (GWRBasic.cpp:386-438); throws NotSPDError.
    void fit(double bw, bool adaptive, int kernel, bool storeS, FitOutput& out);
    // CRSDistance::maxDistance.
    double maxDistance();
    // GWRBasic::predict (GWRBasic.cpp:130-191, predictSerial/Omp/Cuda): beta at
    // nr prediction locations (nr x 2 column-major) from the data's weights at
    // bandwidth bw, in FP64 with the exact thresholds (both numeric forms);
    // betas: nr x p column-major.  Throws NotSPDError like the reference.
    void predict(int nr, const double* locations, double bw, bool adaptive, int kernel, std::vector<double>& betas);
    // Golden-section bandwidth search on the device-resident data
    // (BandwidthSelector::optimize); returns the chosen bandwidth and fills
    // record with (bandwidth, criterion).
    double golden(bool adaptive, int kernel, int crit, double lower, double upper, std::map<double, double>& record);
    // Forget the per-dataset caches (order statistics, distance histograms,
    // thresholds, the distance cache's contents) so the next search
    // recomputes everything.
    void clearCaches();
    // Distance cache of the mixed geographic contraction (the FP32 squared
    // distance of every pair, n^2 x 4 bytes: 160 GB at n = 200,000).  One
    // buffer per device is shared by the engines on it: the engine that
    // uses it last owns its contents, and it is freed with its owner or by
    // releaseDistanceCache().  limit < 0: automatic (used when the device
    // keeps max(16 GB, 1/8 of its memory) free beside it); 0: never; > 0: at
    // most that many bytes.
    void setDistanceCacheLimit(long long bytes) { d2c_limit_bytes_ = bytes; }
    void releaseDistanceCache();
    bool distanceCacheActive() const;
    // CUDA events on the engine stream (slots 0..7) for device timing.
    void recordEvent(int slot);
    float elapsedMs(int a, int b);
    // indepVarsSelectionCriterion (GWRBasic.cpp:309-346): AICc of the model
    // on the given columns with every weight equal to one; DBL_MAX on failure.
    double globalCriterion(const std::vector<int>& cols);
    // Per-row adaptive thresholds (fixbw) in original order, for tests.
    void thresholds(double bw, bool adaptive, std::vector<double>& out);

    // Event timings and counters; `phases` adds the contraction's clock64 phase
    // counters (instrumented kernels, for profiling only).
    void enableStats(bool on, bool phases = false)
    {
        stats_on_ = on;
        phases_on_ = on && phases;
    }
    // Counters and event timings; resolving them waits for the recorded
    // events, never for anything during a fit.
    EngineStats& stats();
    void resetStats();
    cudaStream_t stream() const { return stream_; }
    void synchronize();

    // tcgen05 self-test: D[128 x N] = A[128 x 32] B[N x 32]^T (host arrays).
    void tcSelftest(int N, const float* A, const float* B, float* D);

private:
    friend class BatchEngine;  // builds per-segment kernel arguments over the engine's device data
    void ensureMixed();
    void buildProxy();
    void contractMixed(double* G, int ldg, int mcols, double bw, bool adaptive, int kernel, bool exclude_self,
                       int wpow);
    const float* ensureDistanceCache();  // called with the device cache's lock held
    float* acquireDistanceCache();       // likewise
    void computeThresholds(double bw, bool adaptive);
    const double* thrPtr(bool adaptive) const { return adaptive ? thr_.get() : nullptr; }
    void contract(const double* Z, int mcols, double* G, int ldg, double bw, bool adaptive, int kernel,
                  bool exclude_self, int wpow);
    void solve(int mode, double bw, bool adaptive, int kernel, double out[4]);
    void refine(double bw, bool adaptive, int kernel, double out[4]);
    DevPoints points() const;
    void copyOut(const double* dev, int cols, std::vector<double>& out);
    double* ainv_out_ = nullptr;  // fit-mode solve: where to store A_i^-1 (fitDevice)

    int device_ = 0;
    int num_sms_ = 0;
    cudaStream_t stream_ = nullptr;
    int n_ = 0, p_ = 0, m_ = 0, mm_ = 0;
    bool geographic_ = false;
    int precision_ = kFP64;
    int flush_tiles_ = 64;
    unsigned tc_wait_limit_ = 0;
    double dlo_ = 0.0, dhi_ = 0.0;
    std::vector<int> perm_;  // sorted position -> original index
    std::vector<double> hx_, hy_, hu_, hv_;  // host copies in sorted order
    std::vector<double> he_;                 // geographic: unit vectors in sorted order (3 x n)

    DevBuf<double> u_, v_, uR_, vR_, e_, x_, y_, z_, g_, g2_;  // e_: unit vectors (geographic)
    DevBuf<double> thr_, sel0_, sel1_;
    // order statistics already computed, by rank: brackets for new ranks
    struct RankStat {
        unsigned rank;
        bool exact;
        DevBuf<double> v;
    };
    std::vector<std::unique_ptr<RankStat>> ranks_;
    std::vector<std::unique_ptr<RankStat>> rank_pool_;  // recycled order-statistic buffers
    void recycleRanks()
    {
        for (auto& r : ranks_) rank_pool_.push_back(std::move(r));
        ranks_.clear();
    }
    long long hist_limit_bytes_ = -1;  // histogram cache limit; -1: a quarter of the free memory
    DevBuf<unsigned> hist_;    // per-row histograms of proxy distances (n x 4096)
    DevBuf<unsigned> hcoarse_; // their cumulative counts per 64-bin segment (n x 64)
    bool hist_tried_ = false, hist_valid_ = false;
    const double* orderStatistic(unsigned rank);
    DevBuf<float4> tbsel_;     // FP32 bounds of the 32-point tiles (select, mixed kernels)
    DevBuf<float4> tb16_;      // FP32 bounds of the 16-point tiles (FP64 kernels)
    DevBuf<float> tile_thr16_;
    DevBuf<int> sel_err_;
    double sel_eps_ = 0.0, sel_delta_ = 0.0;
    DevBuf<double> beta_, sii_, resid_, vvec_, bse_, qdiag_, S_;
    DevBuf<double> partials_, sums_;
    DevBuf<double> gall_, gall_part_, gsub_, xsub_;
    bool gall_valid_ = false;
    DevBuf<TileBox> tiles_;
    DevBuf<TileCap> caps_;      // geographic bounds of the 16-point tiles
    int refine_steps_ = 1;
    bool refine_search_ = false;

    // mixed-precision state (built on first use): X~ = (X - mu) / s, y~ likewise
    bool mixed_ready_ = false;
    int npad_ = 0, ntiles32_ = 0, intercept_col_ = -1;
    double uc_ = 0.0, vc_ = 0.0, slack_ = 0.0;  // planar frame of the FP32 records and tile bounds
    std::vector<double> mu_, sc_;  // per column mean (0 if not centred) and scale
    double mu_y_ = 0.0, s_y_ = 1.0;
    DevBuf<double> xs_, ys_, zs_;
    DevBuf<unsigned char> zimg_;
    DevBuf<float4> pts32_;
    DevBuf<TileBox> boxes32_;
    DevBuf<TileCap> caps32_;
    DevBuf<double> rvec_;
    DevBuf<float2> acc_;
    DevBuf<float> stage_;
    DevBuf<int> fill_scratch_;  // work items of the symmetric distance-cache fill
    DevBuf<float> thr32_;
    DevBuf<int> err_;
    long long d2c_limit_bytes_ = -1;
    bool d2c_valid_ = false;  // this engine's dataset is in the device cache (while it owns it)
    DevBuf<unsigned long long> tile_count_;
    DevBuf<unsigned long long> tc_prof_;  // phase cycles of the contraction (stats)
    // prediction points (Hilbert order): FP64 coordinates, FP32 records, 16-point
    // tile bounds, thresholds, normal equations and coefficients
    DevBuf<double> pf_u_, pf_v_, pf_uR_, pf_vR_, pf_e_, pf_thr_, pf_d0_, pf_d1_, pf_g_, pf_beta_;
    DevBuf<float4> pf_pts_, pf_tb16_;
    DevBuf<float4> stb_;  // bounds of the 1024-point super-tiles (select)
    // event pairs recorded around timed launches, resolved by stats()
    struct PendingTiming {
        cudaEvent_t e0, e1;
        int kind;  // 0: contraction, 1: select
    };
    std::vector<PendingTiming> pending_;
    bool counters_dirty_ = false;
    cudaEvent_t timerBegin();
    void timerEnd(cudaEvent_t e0, int kind);  // processed-tile counter of the contraction (stats)
    DevBuf<double> tinv_, tvec_;   // transform of the fit's covariance diagonal
    DevBuf<unsigned long long> key_;  // maxDistance: fast and exact maxima as ordered keys
    DevBuf<double> rowmax_;           // maxDistance: per-row maxima of the fast pass (geographic)
    double* host_sums_ = nullptr;  // pinned

    bool thr_valid_ = false;
    double thr_bw_ = 0.0;
    int thr_prec_ = -1;

    bool stats_on_ = false, phases_on_ = false;
    EngineStats stats_;
    cudaEvent_t events_[8] = {};
};

}  // namespace gwgpu
