// gwrbasic.cpp -- gwm::GWRBasic drop-in: the orchestration of GWRBasic::fit
// (GWRBasic.cpp:36-128), BandwidthSelector::optimize
// (BandwidthSelector.cpp:6-95) and VariableForwardSelector
// (VariableForwardSelector.cpp:9-91) on the host, every per-location
// computation on the GPU engine.
#include "../../include/gwmodel_gb300/GWRBasic.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <stdexcept>

#include "engine.h"
#include "golden.h"

namespace gwm {

namespace {
const char* kFile = "gwrbasic.cpp";
}

struct GWRBasic::Impl {
    std::unique_ptr<gwgpu::Engine> engine;
    int device = -1;
};

#define GW_LOG(LEVEL, MSG) mTelegram->print((MSG), ITelegram::LogLevel::LEVEL, __func__, kFile)
#define GW_STAGE(NAME) GW_LOG(LOG_INFO, std::string("#stage ") + (NAME))
#define GW_STOP_RETURN(REVAL)               \
    if (mTelegram->stop()) {                \
        mStatus = Status::Terminated;       \
        return (REVAL);                     \
    }

GWRBasic::GWRBasic() : mTelegram(new Logger()), mImpl(new Impl()) {}

GWRBasic::GWRBasic(const mat& x, const vec& y, const mat& coords, const SpatialWeight& spatialWeight,
                   bool hasHatMatrix, bool hasIntercept)
    : mX(x), mCoords(coords), mY(y), mSpatialWeight(spatialWeight), mHasIntercept(hasIntercept),
      mHasHatMatrix(hasHatMatrix), mTelegram(new Logger()), mImpl(new Impl())
{
}

GWRBasic::~GWRBasic() = default;

// GWRBasic::setBandwidthSelectionCriterion (GWRBasic.cpp:904-940): every
// ParallelType maps to the same GPU criterion here.
void GWRBasic::setBandwidthSelectionCriterion(const BandwidthSelectionCriterionType& criterion)
{
    mBandwidthSelectionCriterion = criterion;
    mCriterionFunction = criterion;
}

// GWRBasic::setParallelType (GWRBasic.cpp:942-975).
void GWRBasic::setParallelType(const ParallelType& type)
{
    if (type & parallelAbility()) {
        mParallelType = type;
        setBandwidthSelectionCriterion(mBandwidthSelectionCriterion);
    }
}

// GWRBasic::isValid (GWRBasic.cpp:977-990) with GWRBase::isValid.
bool GWRBasic::isValid()
{
    if (!(mX.n_cols > 0)) return false;
    if (!(mX.n_rows == mY.n_rows && mX.n_rows == mCoords.n_rows)) return false;
    if (mCoords.n_cols != 2) return false;
    return mSpatialWeight.weight()->bandwidth() > 0;
}

static std::string infoBandwidthCriterion(const BandwidthWeight& w)
{
    return std::string("#bandwidth-criterion ") + (w.adaptive() ? "adaptive" : "fixed") + ",criterion";
}

static std::string infoBandwidthCriterion(const BandwidthWeight& w, double value)
{
    if (w.adaptive())
        return std::string("#bandwidth-criterion ") + std::to_string(int(w.bandwidth())) + "," + std::to_string(value);
    return std::string("#bandwidth-criterion ") + std::to_string(w.bandwidth()) + "," + std::to_string(value);
}

static std::string infoVariableCriterion(const std::vector<std::size_t>& vars, double value)
{
    std::string s = "#variable-criterion ";
    for (std::size_t i = 0; i < vars.size(); i++) s += (i ? "+" : "") + std::to_string(vars[i]);
    return s + "," + std::to_string(value);
}

static std::vector<int> index2cols(const std::vector<std::size_t>& index, bool hasIntercept)
{
    std::vector<int> cols;
    if (hasIntercept) cols.push_back(0);
    for (std::size_t v : index) cols.push_back((int)v);
    return cols;
}

// bandwidthSizeCriterion{AIC,CV}Cuda (GWRBasic.cpp:709-836).
double GWRBasic::bandwidthCriterion(const BandwidthWeight& w)
{
    if (mTelegram->stop()) {
        mStatus = Status::Terminated;
        return DBL_MAX;
    }
    double value = mImpl->engine->criterion(w.bandwidth(), w.adaptive(), (int)w.kernel(),
                                            mCriterionFunction == CV ? gwgpu::kCV : gwgpu::kAIC);
    if (mStatus == Status::Success && value < DBL_MAX && std::isfinite(value)) {
        GW_LOG(LOG_INFO, infoBandwidthCriterion(w, value));
        mTelegram->progress(std::exp(-std::abs(mBandwidthLastCriterion - value)), __func__, kFile);
        mBandwidthLastCriterion = value;
        return value;
    }
    if (value == DBL_MAX) GW_LOG(LOG_ERR, "Cuda failed to get the inverse of matrix");
    return DBL_MAX;
}

// indepVarsSelectionCriterionCuda (GWRBasic.cpp:838-900): w == 1.
double GWRBasic::indepVarsCriterion(const std::vector<std::size_t>& vars)
{
    if (mTelegram->stop()) {
        mStatus = Status::Terminated;
        return DBL_MAX;
    }
    double value = mImpl->engine->globalCriterion(index2cols(vars, mHasIntercept));
    mTelegram->progress(++mIndepVarSelectionProgressCurrent, mIndepVarSelectionProgressTotal, __func__, kFile);
    if (mStatus == Status::Success && value < DBL_MAX && std::isfinite(value)) {
        GW_LOG(LOG_INFO, infoVariableCriterion(vars, value));
        return value;
    }
    return DBL_MAX;
}

mat GWRBasic::fit()
{
    GW_STAGE("Initializing");
    const std::size_t nDp = mCoords.n_rows;
    std::size_t nVars = mX.n_cols;
    if (mCoords.n_cols != 2) throw std::runtime_error("The dimension of data points or focus points is not 2.");
    if (mX.n_rows != nDp || mY.n_rows != nDp) throw std::runtime_error("X, y and coords differ in rows");
    const bool geographic = mSpatialWeight.distance()->geographic();
    if (!mImpl->engine || mImpl->device != mGpuId) {
        mImpl->engine.reset(new gwgpu::Engine(mGpuId));
        mImpl->device = mGpuId;
    }
    gwgpu::Engine& eng = *mImpl->engine;
    eng.setPrecision((int)mPrecision);
    eng.setData((int)nDp, (int)nVars, mX.memptr(), mY.memptr(), mCoords.memptr(), geographic);
    GW_STOP_RETURN(mat(nDp, nVars));

    if (mIsAutoselectIndepVars) {
        GW_STAGE("Independent variable selection");
        std::vector<std::size_t> indep_vars;
        for (std::size_t i = (mHasIntercept ? 1 : 0); i < mX.n_cols; i++) indep_vars.push_back(i);
        const std::size_t k = indep_vars.size();
        mIndepVarSelectionProgressTotal = (k + 1) * k / 2;
        mIndepVarSelectionProgressCurrent = 0;
        GW_LOG(LOG_INFO, "#variable-criterion variables,criterion");
        // VariableForwardSelector::optimize (VariableForwardSelector.cpp:9-42)
        std::vector<std::size_t> curIndex, restIndex;
        for (std::size_t i = 0; i < k; i++) restIndex.push_back(i);
        std::vector<std::pair<std::vector<std::size_t>, double>> models;
        auto toVars = [&](const std::vector<std::size_t>& idx) {
            std::vector<std::size_t> v;
            for (std::size_t i : idx) v.push_back(indep_vars[i]);
            return v;
        };
        for (std::size_t i = 0; i < k && mStatus == Status::Success; i++) {
            std::vector<double> crit(restIndex.size(), DBL_MAX);
            for (std::size_t j = 0; j < restIndex.size() && mStatus == Status::Success; j++) {
                curIndex.push_back(restIndex[j]);
                double aic = indepVarsCriterion(toVars(curIndex));
                crit[j] = aic;
                models.push_back({curIndex, aic});
                curIndex.pop_back();
            }
            std::size_t best = std::min_element(crit.begin(), crit.end()) - crit.begin();
            curIndex.push_back(restIndex[best]);
            restIndex.erase(restIndex.begin() + best);
        }
        if (mStatus == Status::Success) {
            // sort(): each forward step's block by criterion, descending (:52-64)
            std::size_t tag = 0;
            for (std::size_t size = k; size > 0; size--) {
                std::stable_sort(models.begin() + tag, models.begin() + tag + size,
                                 [](const auto& a, const auto& b) { return a.second > b.second; });
                tag += size;
            }
            // select(): the last model whose predecessor is worse by >= threshold (:66-76)
            auto chosen = models.back();
            for (std::size_t i = models.size() - 1; i > 0; i--) {
                if (models[i - 1].second - models[i].second >= mIndepVarSelectionThreshold) {
                    chosen = models[i];
                    break;
                }
            }
            mSelectedIndepVars = toVars(chosen.first);
            mIndepVarsSelectionCriterionList.clear();
            for (auto& m : models) mIndepVarsSelectionCriterionList.push_back({toVars(m.first), m.second});
            if (!mSelectedIndepVars.empty()) {
                std::vector<int> cols = index2cols(mSelectedIndepVars, mHasIntercept);
                mat xs(nDp, cols.size());
                for (std::size_t c = 0; c < cols.size(); c++)
                    for (std::size_t i = 0; i < nDp; i++) xs(i, c) = mX(i, cols[c]);
                mX = xs;
                nVars = mX.n_cols;
                eng.setData((int)nDp, (int)nVars, mX.memptr(), mY.memptr(), mCoords.memptr(), geographic);
            }
        }
        GW_STOP_RETURN(mat(nDp, nVars));
    }

    if (mIsAutoselectBandwidth) {
        GW_STAGE("Bandwidth selection");
        BandwidthWeight bw0 = *mSpatialWeight.weight();
        const bool adaptive = bw0.adaptive();
        double lower = mGoldenLowerBounds.value_or(adaptive ? 20 : 0.0);
        double upper = mGoldenUpperBounds.value_or(adaptive ? (double)nDp : eng.maxDistance());
        GW_LOG(LOG_INFO, infoBandwidthCriterion(bw0));
        // BandwidthSelector::optimize (BandwidthSelector.cpp:6-81)
        std::map<double, double> record;
        BandwidthWeight w = bw0;
        double xopt = 0.0;
        const bool chosen = gwgpu::golden_section(
            lower, upper, adaptive,
            [&](double b) {
                w.setBandwidth(b);
                return bandwidthCriterion(w);
            },
            [&] { return mStatus == Status::Success; }, xopt, record);
        if (chosen) {
            BandwidthWeight wopt;
            wopt.setKernel(bw0.kernel());
            wopt.setAdaptive(bw0.adaptive());
            wopt.setBandwidth(xopt);
            mSpatialWeight.setWeight(wopt);
            mBandwidthSelectionCriterionList.assign(record.begin(), record.end());
        }
        GW_STOP_RETURN(mat(nDp, nVars));
    }

    GW_STAGE("Model fitting");
    const BandwidthWeight& bw = *mSpatialWeight.weight();
    const bool storeS = mHasHatMatrix && nDp < 8192;  // isStoreS (GWRBasic.h:708)
    GW_STOP_RETURN(mat(nDp, nVars));
    gwgpu::FitOutput out;
    try {
        eng.fit(bw.bandwidth(), bw.adaptive(), (int)bw.kernel(), storeS, out);
    } catch (const gwgpu::NotSPDError& e) {
        GW_LOG(LOG_ERR, "Cuda failed to get the inverse of matrix");
        throw std::runtime_error("Cuda failed to get the inverse of matrix");
    }
    mTelegram->progress(nDp, nDp, __func__, kFile);
    mBetas = mat(nDp, nVars, out.betas.data());
    mBetasSE = mat(nDp, nVars, out.betasSE.data());
    mSHat = vec(2, 1, out.shat);
    mQDiag = vec(nDp, 1, out.qdiag.data());
    mS = mat((std::size_t)out.sRows, nDp, out.S.data());
    GW_STOP_RETURN(mat(nDp, nVars));

    GW_STAGE("Model Diagnostic");
    // CalcDiagnostic (GWRBasic.cpp:21-34)
    const double n = (double)nDp;
    double rss = 0.0, ymean = 0.0;
    for (std::size_t i = 0; i < nDp; i++) {
        double fit = 0.0;
        for (std::size_t k = 0; k < nVars; k++) fit += mBetas(i, k) * mX(i, k);
        double r = mY(i) - fit;
        rss += r * r;
        ymean += mY(i);
    }
    ymean /= n;
    double yss = 0.0;
    for (std::size_t i = 0; i < nDp; i++) yss += (mY(i) - ymean) * (mY(i) - ymean);
    const double trS = mSHat(0), trStS = mSHat(1);
    mDiagnostic.RSS = rss;
    mDiagnostic.AIC = n * std::log(rss / n) + n * std::log(2 * M_PI) + n + trS;
    mDiagnostic.AICc = n * std::log(rss / n) + n * std::log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
    mDiagnostic.EDF = n - 2 * trS + trStS;
    mDiagnostic.ENP = 2 * trS - trStS;
    mDiagnostic.RSquare = 1 - rss / yss;
    mDiagnostic.RSquareAdjust = 1 - (1 - mDiagnostic.RSquare) * (n - 1) / (mDiagnostic.EDF - 1);
    // betasSE = sqrt(sigmaHat * betasSE) (GWRBasic.cpp:105-106); the local R2
    // loop that follows in the reference stores nothing and is not repeated.
    const double sigmaHat = rss / (n - 2 * trS + trStS);
    for (std::size_t e = 0; e < mBetasSE.n_elem(); e++) mBetasSE.memptr()[e] = std::sqrt(sigmaHat * mBetasSE.memptr()[e]);
    return mBetas;
}

// GWRBasic::predict (GWRBasic.cpp:130-155) with predictSerial/Omp/Cuda
// (GWRBasic.cpp:165-191, 665-707): the stages, stop checks and the zero
// matrix of the reference's stop path (nDp x nVars) are kept.
mat GWRBasic::predict(const mat& locations)
{
    GW_STAGE("Initialization");
    const std::size_t nDp = mCoords.n_rows, nVars = mX.n_cols, nRp = locations.n_rows;
    if (mCoords.n_cols != 2 || locations.n_cols != 2)
        throw std::runtime_error("The dimension of data points or focus points is not 2.");
    if (mX.n_rows != nDp || mY.n_rows != nDp) throw std::runtime_error("X, y and coords differ in rows");
    const bool geographic = mSpatialWeight.distance()->geographic();
    if (!mImpl->engine || mImpl->device != mGpuId) {
        mImpl->engine.reset(new gwgpu::Engine(mGpuId));
        mImpl->device = mGpuId;
    }
    gwgpu::Engine& eng = *mImpl->engine;
    eng.setPrecision((int)mPrecision);
    eng.setData((int)nDp, (int)nVars, mX.memptr(), mY.memptr(), mCoords.memptr(), geographic);
    GW_STOP_RETURN(mat(nDp, nVars));

    GW_STAGE("Prediction");
    const BandwidthWeight& bw = *mSpatialWeight.weight();
    std::vector<double> b;
    try {
        eng.predict((int)nRp, locations.memptr(), bw.bandwidth(), bw.adaptive(), (int)bw.kernel(), b);
    } catch (const gwgpu::NotSPDError& e) {
        GW_LOG(LOG_ERR, e.what());
        throw std::runtime_error(e.what());
    }
    mTelegram->progress(nRp, nRp, __func__, kFile);
    mBetas = mat(nRp, nVars, b.data());
    GW_STOP_RETURN(mat(nDp, nVars));
    return mBetas;
}

}  // namespace gwm
