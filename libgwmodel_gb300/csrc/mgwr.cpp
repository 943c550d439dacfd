// mgwr.cpp -- gwm::GWRMultiscale drop-in: GWRMultiscale::fit and backfitting
// (GWRMultiscale.cpp:68-317) orchestrated on the host; every criterion, fit
// and hat-matrix product runs on the GPU.
//
// One engine holds the coordinates in Hilbert order for the whole fit.  The
// per-variable problems (x_k, y_i) and the all-variable problem swap only X
// and y (Engine::setVariables), so the distance caches (adaptive thresholds,
// order statistics) built by one bandwidth search serve every later search.
//
// Hat matrix (GWRMultiscale.cpp:216-224, 296-301): S0, SA_k (k < p) and the
// scratch T = SA_k - S0 are n x n FP64 matrices resident on the device in the
// sorted order.  The update SA_k = S T + S = S (T + I) is one fused kernel that
// forms S's entries w_ij v_i x_j on the fly (S is never stored): for a compact
// kernel (bisquare, tricube, boxcar) it visits only the rows of T within the
// variable's bandwidth (2 n k n flops instead of 2 n^3); gaussian and
// exponential kernels visit every row (the dense 2 n^3 product).  tr(S0) and
// tr(S0^T S0) are reduced on the device at the end.
#include "../../include/gwmodel_gb300/GWRMultiscale.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <stdexcept>

#include "engine.h"
#include "golden.h"
#include "gw_kernels.h"

namespace gwm {

namespace {
const char* kFile = "mgwr.cpp";

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

std::string strjoin(const std::string& sep, const std::vector<std::string>& parts)
{
    std::string s;
    for (std::size_t i = 0; i < parts.size(); i++) s += (i ? sep : "") + parts[i];
    return s;
}
}  // namespace

struct GWRMultiscale::Impl {
    std::unique_ptr<gwgpu::Engine> engine;
    int device = -1;
    // hat-matrix state
    gwgpu::DevBuf<double> S0, SA, T, ainv, partials, sums;
    void releaseHat()
    {
        S0.release();
        SA.release();
        T.release();
        ainv.release();
    }
};

#define GW_LOG(LEVEL, MSG) mTelegram->print((MSG), ITelegram::LogLevel::LEVEL, __func__, kFile)
#define GW_STAGE(NAME) GW_LOG(LOG_INFO, std::string("#stage ") + (NAME))
#define GW_BACKFITTING(MSG) GW_LOG(LOG_INFO, std::string("#back-fitting ") + (MSG))
#define GW_STOP_RETURN(REVAL)         \
    if (mTelegram->stop()) {          \
        mStatus = Status::Terminated; \
        return (REVAL);               \
    }

GWRMultiscale::GWRMultiscale() : mTelegram(new Logger()), mImpl(new Impl()) {}

GWRMultiscale::GWRMultiscale(const mat& x, const vec& y, const mat& coords,
                             const std::vector<SpatialWeight>& spatialWeights)
    : mX(x), mCoords(coords), mY(y), mSpatialWeights(spatialWeights), mTelegram(new Logger()), mImpl(new Impl())
{
}

GWRMultiscale::~GWRMultiscale() = default;

void GWRMultiscale::setSpatialWeights(const std::vector<SpatialWeight>& sw) { mSpatialWeights = sw; }

// GWRMultiscale.cpp:1485-1510: the size must match the columns of X.
void GWRMultiscale::setBandwidthInitilize(const std::vector<BandwidthInitilizeType>& v)
{
    if (v.size() != mX.n_cols) throw std::length_error("BandwidthInitilize size do not match indepvars");
    mBandwidthInitilize = v;
}

void GWRMultiscale::setBandwidthSelectionApproach(const std::vector<BandwidthSelectionCriterionType>& v)
{
    if (v.size() != mX.n_cols) throw std::length_error("bandwidthSelectionApproach size do not match indepvars");
    mBandwidthSelectionApproach = v;
}

// GWRMultiscale::isValid (GWRMultiscale.cpp:318-360).
bool GWRMultiscale::isValid()
{
    if (!(mX.n_cols > 0)) return false;
    const std::size_t p = mX.n_cols;
    if (mSpatialWeights.size() != p || mBandwidthInitilize.size() != p || mBandwidthSelectionApproach.size() != p ||
        mPreditorCentered.size() != p || mBandwidthSelectThreshold.size() != p)
        return false;
    for (std::size_t i = 0; i < p; i++) {
        const BandwidthWeight* bw = mSpatialWeights[i].weight();
        if (mBandwidthInitilize[i] == Specified || mBandwidthInitilize[i] == Initial) {
            if (bw->adaptive() ? bw->bandwidth() <= 1 : bw->bandwidth() < 0.0) return false;
        }
    }
    return true;
}

// GWRMultiscale::CalcDiagnostic (GWRMultiscale.cpp:41-66).
RegressionDiagnostic GWRMultiscale::CalcDiagnostic(const mat& x, const vec& y, double trS, double trStS, double RSS)
{
    const std::size_t n_ = x.n_rows;
    const double n = (double)n_;
    double mean = 0.0;
    for (std::size_t i = 0; i < n_; i++) mean += y(i);
    mean /= n;
    double tss = 0.0;
    for (std::size_t i = 0; i < n_; i++) tss += (y(i) - mean) * (y(i) - mean);
    RegressionDiagnostic d{};
    const double r2 = 1 - RSS / tss;
    const double enp = 2 * trS - trStS, edf = n - 2 * trS + trStS;
    d.RSS = RSS;
    d.AIC = 0.0;
    d.AICc = n * std::log(RSS / n) + n * std::log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
    d.ENP = enp;
    d.EDF = edf;
    d.RSquare = r2;
    d.RSquareAdjust = 1 - (1 - r2) * (n - 1) / (edf - 1);
    return d;
}

static std::string infoBandwidthCriterion(const BandwidthWeight& w)
{
    return std::string("#bandwidth-criterion ") + (w.adaptive() ? "adaptive" : "fixed") + ",criterion";
}

// bandwidthSizeCriterion{All,Var}{CV,AIC}Cuda (GWRMultiscale.cpp:1142-1394):
// the engine holds the problem of the current search (all variables, or one
// variable against its partial response).
double GWRMultiscale::bandwidthCriterion(const BandwidthWeight& w, int approach)
{
    if (mTelegram->stop()) {
        mStatus = Status::Terminated;
        return DBL_MAX;
    }
    double value = mImpl->engine->criterion(w.bandwidth(), w.adaptive(), (int)w.kernel(),
                                            approach == CV ? gwgpu::kCV : gwgpu::kAIC);
    mCounters.criterionEvals++;
    if (value < DBL_MAX && std::isfinite(value)) {
        if (w.adaptive())
            GW_LOG(LOG_INFO, std::string("#bandwidth-criterion ") + std::to_string(int(w.bandwidth())) + "," +
                                 std::to_string(value));
        else
            GW_LOG(LOG_INFO,
                   std::string("#bandwidth-criterion ") + std::to_string(w.bandwidth()) + "," + std::to_string(value));
        mTelegram->progress(std::exp(-std::abs(mBandwidthLastCriterion - value)), __func__, kFile);
        mBandwidthLastCriterion = value;
        return value;
    }
    if (value == DBL_MAX) GW_LOG(LOG_ERR, "Cuda failed to get the inverse of matrix");
    return DBL_MAX;
}

// BandwidthSelector::optimize with the bounds of GWRMultiscale.cpp:118-119,
// 141-142, 256-257 for variable var's weight (or the initial weight, all).
// Returns false when the search stopped on a cancelled status: out keeps the
// starting weight, as optimize() returns mBandwidth.
bool GWRMultiscale::selectBandwidth(std::size_t var, bool all, double lower, double upper, BandwidthWeight& out)
{
    const BandwidthWeight w0 = *mSpatialWeights[var].weight();
    const int approach = mBandwidthSelectionApproach[all ? 0 : var];
    std::map<double, double> record;
    double xopt = w0.bandwidth();
    BandwidthWeight probe = w0;
    const double t0 = now_s();
    struct Clock {
        double t0;
        double& acc;
        ~Clock() { acc += now_s() - t0; }
    } clock{t0, mCounters.searchSeconds};
    bool ok = gwgpu::golden_section(
        lower, upper, w0.adaptive(),
        [&](double b) {
            probe.setBandwidth(b);
            return bandwidthCriterion(probe, approach);
        },
        [&] { return mStatus == Status::Success; }, xopt, record);
    out = w0;
    if (ok) out.setBandwidth(xopt);
    return ok;
}

mat GWRMultiscale::fit()
{
    GW_STAGE("Initializing");
    const std::size_t n = mX.n_rows, p = mX.n_cols;
    if (p < 1) throw std::invalid_argument("GWRMultiscale needs at least one independent variable");
    if (mY.n_rows != n || mCoords.n_rows != n || mCoords.n_cols != 2)
        throw std::invalid_argument("x, y and coords must have the same number of rows (coords n x 2)");
    if (mSpatialWeights.size() != p) throw std::length_error("spatialWeights size do not match indepvars");
    if (mBandwidthInitilize.size() != p) throw std::length_error("BandwidthInitilize size do not match indepvars");
    if (mBandwidthSelectionApproach.size() != p)
        throw std::length_error("bandwidthSelectionApproach size do not match indepvars");
    if (mPreditorCentered.size() != p) throw std::length_error("preditorCentered size do not match indepvars");
    if (mBandwidthSelectThreshold.size() != p)
        throw std::length_error("bandwidthSelectThreshold size do not match indepvars");
    const bool geographic = mSpatialWeights[0].distance()->geographic();
    for (const auto& sw : mSpatialWeights)
        if (sw.distance()->geographic() != geographic)
            throw std::invalid_argument("every spatial weight must use the same CRSDistance");
    mStatus = Status::Success;
    mBandwidthLastCriterion = DBL_MAX;
    mIterations = 0;
    mCounters = Counters();
    if (!mImpl->engine || mImpl->device != mGpuId) {
        mImpl->engine.reset(new gwgpu::Engine(mGpuId));
        mImpl->device = mGpuId;
    }
    gwgpu::Engine& eng = *mImpl->engine;
    eng.resetStats();
    eng.setPrecision(mPrecision == Precision::Mixed ? gwgpu::kMixed : gwgpu::kFP64);
    GW_STOP_RETURN(mat(n, p, 0.0));

    // centring of the predictors (:90-99)
    mat x = mX;
    for (std::size_t k = mHasIntercept ? 1 : 0; k < p; k++) {
        if (!mPreditorCentered[k]) continue;
        double m = 0.0;
        for (std::size_t i = 0; i < n; i++) m += x(i, k);
        m /= (double)n;
        for (std::size_t i = 0; i < n; i++) x(i, k) -= m;
    }
    auto col = [&](std::size_t k) { return x.memptr() + k * n; };
    eng.setData((int)n, 1, col(0), mY.memptr(), mCoords.memptr(), geographic);
    const double maxDist = eng.maxDistance();
    auto lowerOf = [&](const BandwidthWeight& w) {
        return mGoldenLowerBounds.value_or(w.adaptive() ? (double)mAdaptiveLower : maxDist / 5000.0);
    };
    auto upperOf = [&](const BandwidthWeight& w) { return mGoldenUpperBounds.value_or(w.adaptive() ? (double)n : maxDist); };
    GW_STOP_RETURN(mat(n, p, 0.0));

    // initial bandwidths of the variables, against y (:104-133)
    GW_STAGE("Calculating initial bandwidths");
    std::vector<BandwidthInitilizeType> init = mBandwidthInitilize;
    for (std::size_t k = 0; k < p && mStatus == Status::Success; k++) {
        if (init[k] == Null) {
            eng.setVariables(1, col(k), mY.memptr());
            GW_LOG(LOG_INFO, std::string("#initial-bandwidth ") + std::to_string(k));
            const BandwidthWeight& w0 = *mSpatialWeights[k].weight();
            BandwidthWeight bw;
            selectBandwidth(k, false, lowerOf(w0), upperOf(w0), bw);
            mSpatialWeights[k].setWeight(bw);
            GW_LOG(LOG_INFO, std::string("#initial-bandwidth ") + std::to_string(k) + "," + std::to_string(bw.bandwidth()));
        }
        GW_STOP_RETURN(mat(n, p, 0.0));
    }
    if (mStatus != Status::Success) return mat(n, p, 0.0);

    // initial all-variable bandwidth with the first variable's weight (:135-155)
    GW_STAGE("Calculating initial bandwidth");
    eng.setVariables((int)p, x.memptr(), mY.memptr());
    const BandwidthWeight w0 = *mSpatialWeights[0].weight();
    GW_LOG(LOG_INFO, infoBandwidthCriterion(w0));
    BandwidthWeight initBw;
    selectBandwidth(0, true, lowerOf(w0), upperOf(w0), initBw);
    mInitBandwidth = initBw.bandwidth();
    GW_STOP_RETURN(mat(n, p, 0.0));

    // hat-matrix storage (:157-163)
    Impl& I = *mImpl;
    const std::size_t nn = n * n;
    if (mHasHatMatrix) {
        const double need = 8.0 * (double)nn * (double)(p + 2) + 8.0 * (double)n * p * p;
        size_t freeb = 0, total = 0;
        gwgpu::check(cudaMemGetInfo(&freeb, &total), "cudaMemGetInfo");
        const double held = (double)(I.S0.capacityBytes() + I.SA.capacityBytes() + I.T.capacityBytes() +
                                     I.ainv.capacityBytes());
        if (need > (double)freeb + held)
            throw std::runtime_error("the hat matrix needs " + std::to_string(need / 1e9) +
                                     " GB of device memory ((p + 2) n x n doubles); disable it with "
                                     "setHasHatMatrix(false)");
        I.S0.alloc(nn);
        I.SA.alloc(nn * p);
        I.T.alloc(nn);
        I.ainv.alloc(n * p * p);
        I.partials.alloc(4096 * 4);
        I.sums.alloc(4);
    }

    // backfitting (:192-317)
    GW_STAGE("Model fitting");
    GW_BACKFITTING("Model fitting with inital bandwidth");
    mat betas(n, p, 0.0);
    {
        double t0 = now_s();
        eng.fitDevice(mInitBandwidth, w0.adaptive(), (int)w0.kernel(), mHasHatMatrix, nullptr,
                      mHasHatMatrix ? I.ainv.get() : nullptr);
        std::vector<double> b;
        eng.betas(b);
        std::copy(b.begin(), b.end(), betas.memptr());
        mCounters.fits++;
        mCounters.fitSeconds += now_s() - t0;
        if (mHasHatMatrix) {
            t0 = now_s();
            eng.betasSE(b);
            mBetasSE = mat(n, p, b.data());
            eng.hatAll(mInitBandwidth, w0.adaptive(), (int)w0.kernel(), I.ainv.get(), I.S0.get(), I.SA.get());
            eng.synchronize();
            mCounters.hatSeconds += now_s() - t0;
        } else {
            mBetasSE = mat();
        }
    }
    GW_STOP_RETURN(mat(n, p, 0.0));

    GW_BACKFITTING("Selecting the optimum bandwidths for each independent variable");
    auto fitted_resid = [&](vec& resid) {
        for (std::size_t i = 0; i < n; i++) {
            double f = 0.0;
            for (std::size_t k = 0; k < p; k++) f += betas(i, k) * x(i, k);
            resid(i, 0) = mY(i) - f;
        }
    };
    std::vector<std::size_t> bwChangeNo(p, 0);
    vec resid(n, 1), yi(n, 1);
    fitted_resid(resid);
    double RSS0 = 0.0, RSS1 = DBL_MAX, criterion = DBL_MAX;
    for (std::size_t i = 0; i < n; i++) RSS0 += resid(i) * resid(i);
    for (std::size_t iteration = 1; iteration <= mMaxIteration && criterion > mCriterionThreshold; iteration++) {
        if (mTelegram->stop()) {
            mStatus = Status::Terminated;
            break;
        }
        GW_BACKFITTING("#iteration " + std::to_string(iteration));
        for (std::size_t k = 0; k < p; k++) {
            if (mTelegram->stop()) {
                mStatus = Status::Terminated;
                break;
            }
            for (std::size_t i = 0; i < n; i++) yi(i, 0) = resid(i) + betas(i, k) * x(i, k);
            eng.setVariables(1, col(k), yi.memptr());
            if (init[k] != Specified) {
                GW_BACKFITTING("#variable-bandwidth-selection " + std::to_string(k));
                const BandwidthWeight& bwi0 = *mSpatialWeights[k].weight();
                // mMaxDistances[k] is only filled for Null-initialised variables (:117); it
                // stays 0 for the others
                const double mdk = mBandwidthInitilize[k] == Null ? maxDist : 0.0;
                const double lo = mGoldenLowerBounds.value_or(bwi0.adaptive() ? (double)mAdaptiveLower : mdk / 5000.0);
                const double hi = mGoldenUpperBounds.value_or(bwi0.adaptive() ? (double)n : mdk);
                BandwidthWeight bwi;
                selectBandwidth(k, false, lo, hi, bwi);
                const double b0 = bwi0.bandwidth(), b1 = bwi.bandwidth();
                std::vector<std::string> args{std::to_string(k), std::to_string(b0), std::to_string(b1),
                                              std::to_string(std::abs(b1 - b0))};
                if (std::abs(b1 - b0) > mBandwidthSelectThreshold[k]) {
                    bwChangeNo[k] = 0;
                    args.push_back("false");
                } else {
                    bwChangeNo[k] += 1;
                    if (bwChangeNo[k] >= mBandwidthSelectRetryTimes) {
                        init[k] = Specified;
                        args.push_back("true");
                    } else {
                        args.push_back(std::to_string(bwChangeNo[k]));
                        args.push_back(std::to_string(mBandwidthSelectRetryTimes - bwChangeNo[k]));
                    }
                }
                mSpatialWeights[k].setWeight(bwi);
                GW_BACKFITTING("#variable-bandwidth-selection " + strjoin(",", args));
            }
            if (mStatus != Status::Success) break;

            const BandwidthWeight& wk = *mSpatialWeights[k].weight();
            double t0 = now_s();
            eng.fitDevice(wk.bandwidth(), wk.adaptive(), (int)wk.kernel(), false, nullptr, nullptr);
            std::vector<double> b;
            eng.betas(b);
            for (std::size_t i = 0; i < n; i++) betas(i, k) = b[i];
            mCounters.fits++;
            mCounters.fitSeconds += now_s() - t0;
            if (mHasHatMatrix) {
                t0 = now_s();
                double* SAk = I.SA.get() + k * nn;
                gwgpu::check(gwgpu::launch_mgwr_sub(nn, SAk, I.S0.get(), I.T.get(), eng.stream()), "hat: T");
                eng.hatUpdate(wk.bandwidth(), wk.adaptive(), (int)wk.kernel(), I.T.get(), SAk);
                gwgpu::check(gwgpu::launch_mgwr_post(nn, SAk, nullptr, I.T.get(), I.S0.get(), eng.stream()),
                             "hat: S0");
                eng.synchronize();
                mCounters.hatUpdates++;
                mCounters.hatSeconds += now_s() - t0;
            }
            fitted_resid(resid);
        }
        if (mStatus != Status::Success) break;
        RSS1 = 0.0;
        {
            vec r(n, 1);
            fitted_resid(r);
            for (std::size_t i = 0; i < n; i++) RSS1 += r(i) * r(i);
        }
        criterion = (mCriterionType == CVR) ? std::abs(RSS1 - RSS0) : std::sqrt(std::abs(RSS1 - RSS0) / RSS1);
        GW_BACKFITTING("#backfitting-criterion " + std::to_string(criterion));
        mTelegram->progress(std::exp(-std::abs(criterion - mCriterionThreshold)), __func__, kFile);
        RSS0 = RSS1;
        mIterations = iteration;
    }
    if (mStatus != Status::Success) {
        I.releaseHat();
        mBetas = betas;
        return betas;
    }
    GW_BACKFITTING("Finished");
    mRSS0 = RSS0;

    // diagnostics (:165-180)
    GW_STAGE("Model Diagnostic");
    double trS = 0.0, trStS = 0.0;
    if (mHasHatMatrix) {
        int nb = 0;
        gwgpu::check(gwgpu::launch_mgwr_traces((int)n, I.S0.get(), I.partials.get(), 4096, &nb, eng.stream()),
                     "hat: traces");
        gwgpu::check(gwgpu::launch_reduce_partials(I.partials.get(), nb, I.sums.get(), eng.stream()), "hat: reduce");
        double h[4];
        gwgpu::check(cudaMemcpyAsync(h, I.sums.get(), sizeof(h), cudaMemcpyDeviceToHost, eng.stream()), "D2H");
        eng.synchronize();
        trS = h[0];
        trStS = h[1];
        I.releaseHat();  // (p + 2) n^2 doubles: not held past the fit
    }
    mDiagnostic = CalcDiagnostic(x, mY, trS, trStS, mRSS0);
    // this library's kernels (the DGEMMs are cuBLAS's): the engine's (including
    // the sparse hat updates), plus the two elementwise passes of each hat
    // update and the final trace reduction
    mCounters.kernelLaunches =
        eng.stats().kernel_launches + (mHasHatMatrix ? 2 * (long long)mCounters.hatUpdates + 2 : 0);
    mBetas = betas;
    if (mHasHatMatrix) {
        mBetasTV = mat(n, p, 0.0);
        for (std::size_t e = 0; e < n * p; e++) mBetasTV.memptr()[e] = betas.memptr()[e] / mBetasSE.memptr()[e];
    } else {
        mBetasTV = mat();
    }
    return mBetas;
}

}  // namespace gwm
