// GWRMultiscale.h -- C++ drop-in for gwm::GWRMultiscale (multiscale GWR by
// back-fitting) backed by the GB300 engine.
//
// Same enums, setters, fit() and getters as libgwmodel's GWRMultiscale
// (include/gwmodelpp/GWRMultiscale.h:35-1040, SpatialMultiscaleAlgorithm.h:55-90)
// and the same tagged telegram messages.  Matrices are the column-major
// gwm::mat of GWRBasic.h.  Every fit runs on the GPU whatever ParallelType
// says.  Unlike the reference, every spatial weight must use the same
// CRSDistance (planar or geographic), since one device-resident geometry
// serves all variables.
#pragma once

#include "GWRBasic.h"

namespace gwm {

class GWRMultiscale {
public:
    enum BandwidthInitilizeType { Null, Initial, Specified };
    enum BandwidthSelectionCriterionType { CV, AIC };
    enum BackFittingCriterionType { CVR, dCVR };

    GWRMultiscale();
    GWRMultiscale(const mat& x, const vec& y, const mat& coords, const std::vector<SpatialWeight>& spatialWeights);
    ~GWRMultiscale();
    GWRMultiscale(const GWRMultiscale&) = delete;
    GWRMultiscale& operator=(const GWRMultiscale&) = delete;

    // SpatialAlgorithm / SpatialMultiscaleAlgorithm / IRegressionAnalysis
    void setCoords(const mat& coords) { mCoords = coords; }
    const mat& coords() const { return mCoords; }
    void setDependentVariable(const vec& y) { mY = y; }
    const vec& dependentVariable() const { return mY; }
    void setIndependentVariables(const mat& x) { mX = x; }
    const mat& independentVariables() const { return mX; }
    void setSpatialWeights(const std::vector<SpatialWeight>& sw);
    const std::vector<SpatialWeight>& spatialWeights() const { return mSpatialWeights; }
    bool hasIntercept() const { return mHasIntercept; }
    void setHasIntercept(bool has) { mHasIntercept = has; }

    // GWRMultiscale setters (GWRMultiscale.h:252-530); the vector setters throw
    // std::length_error when the size differs from the number of columns of X.
    void setGoldenUpperBounds(double value) { mGoldenUpperBounds = value; }
    void setGoldenLowerBounds(double value) { mGoldenLowerBounds = value; }
    const std::vector<BandwidthInitilizeType>& bandwidthInitilize() const { return mBandwidthInitilize; }
    void setBandwidthInitilize(const std::vector<BandwidthInitilizeType>& v);
    const std::vector<BandwidthSelectionCriterionType>& bandwidthSelectionApproach() const
    {
        return mBandwidthSelectionApproach;
    }
    void setBandwidthSelectionApproach(const std::vector<BandwidthSelectionCriterionType>& v);
    const std::vector<bool>& preditorCentered() const { return mPreditorCentered; }
    void setPreditorCentered(const std::vector<bool>& v) { mPreditorCentered = v; }
    const std::vector<double>& bandwidthSelectThreshold() const { return mBandwidthSelectThreshold; }
    void setBandwidthSelectThreshold(const std::vector<double>& v) { mBandwidthSelectThreshold = v; }
    bool hasHatMatrix() const { return mHasHatMatrix; }
    void setHasHatMatrix(bool has) { mHasHatMatrix = has; }
    std::size_t bandwidthSelectRetryTimes() const { return mBandwidthSelectRetryTimes; }
    void setBandwidthSelectRetryTimes(std::size_t t) { mBandwidthSelectRetryTimes = t; }
    std::size_t maxIteration() const { return mMaxIteration; }
    void setMaxIteration(std::size_t m) { mMaxIteration = m; }
    BackFittingCriterionType criterionType() const { return mCriterionType; }
    void setCriterionType(const BackFittingCriterionType& t) { mCriterionType = t; }
    double criterionThreshold() const { return mCriterionThreshold; }
    void setCriterionThreshold(double t) { mCriterionThreshold = t; }
    int adaptiveLower() const { return mAdaptiveLower; }
    void setAdaptiveLower(int l) { mAdaptiveLower = l; }

    int parallelAbility() const { return SerialOnly | OpenMP | CUDA; }
    ParallelType parallelType() const { return mParallelType; }
    void setParallelType(const ParallelType& type)
    {
        if (type & parallelAbility()) mParallelType = type;
    }
    void setOmpThreadNum(int threadNum) { mOmpThreadNum = threadNum; }
    void setGPUId(int gpuId) { mGpuId = gpuId; }
    void setGroupSize(std::size_t size) { mGroupLength = size; }
    // Numeric form of the bandwidth searches: FP64 (the drop-in) or the
    // tensor-core criterion; fits and the hat matrix are always FP64.
    void setPrecision(Precision p) { mPrecision = p; }
    Precision precision() const { return mPrecision; }

    // Algorithm
    void setTelegram(std::unique_ptr<ITelegram> telegram) { mTelegram = std::move(telegram); }
    Status status() const { return mStatus; }
    bool isValid();

    mat fit();
    // GWRMultiscale::predict returns zeros of nRp x nVar (GWRMultiscale.h:601).
    mat predict(const mat& locations) const { return mat(locations.n_rows, mX.n_cols, 0.0); }

    // results
    const mat& betas() const { return mBetas; }
    // diag(C C^T) of the initial all-variable fit (hat matrix only).
    const mat& betasSE() const { return mBetasSE; }
    // betas / betasSE (hat matrix only).
    const mat& betasTV() const { return mBetasTV; }
    RegressionDiagnostic diagnostic() const { return mDiagnostic; }
    // The initial all-variable bandwidth (mInitSpatialWeight after fit()).
    double initialBandwidth() const { return mInitBandwidth; }
    // Back-fitting iterations run.
    std::size_t iterations() const { return mIterations; }
    // Work and host wall time of the last fit() by phase: the bandwidth
    // searches, the fits (fitAll / fitVar), and the hat-matrix updates.
    struct Counters {
        std::size_t criterionEvals = 0, fits = 0, hatUpdates = 0;
        long long kernelLaunches = 0;
        double searchSeconds = 0.0, fitSeconds = 0.0, hatSeconds = 0.0;
    };
    const Counters& counters() const { return mCounters; }
    // GWRMultiscale::CalcDiagnostic (GWRMultiscale.cpp:41-66); AIC, which it
    // leaves unset, is 0.
    static RegressionDiagnostic CalcDiagnostic(const mat& x, const vec& y, double trS, double trStS, double RSS);

private:
    struct Impl;
    double bandwidthCriterion(const BandwidthWeight& w, int approach);
    bool selectBandwidth(std::size_t var, bool all, double lower, double upper, BandwidthWeight& out);

    mat mX, mCoords, mBetas, mBetasSE, mBetasTV;
    vec mY;
    std::vector<SpatialWeight> mSpatialWeights;
    std::vector<BandwidthInitilizeType> mBandwidthInitilize;
    std::vector<BandwidthSelectionCriterionType> mBandwidthSelectionApproach;
    std::vector<bool> mPreditorCentered;
    std::vector<double> mBandwidthSelectThreshold;
    std::optional<double> mGoldenUpperBounds, mGoldenLowerBounds;
    std::size_t mBandwidthSelectRetryTimes = 5, mMaxIteration = 500, mIterations = 0;
    BackFittingCriterionType mCriterionType = dCVR;
    double mCriterionThreshold = 1e-6;
    int mAdaptiveLower = 10;
    bool mHasHatMatrix = true, mHasIntercept = true;
    ParallelType mParallelType = SerialOnly;
    int mOmpThreadNum = 8, mGpuId = 0;
    std::size_t mGroupLength = 64;
    Precision mPrecision = Precision::FP64;
    double mBandwidthLastCriterion = DBL_MAX, mInitBandwidth = 0.0, mRSS0 = 0.0;
    RegressionDiagnostic mDiagnostic{};
    Counters mCounters;
    std::unique_ptr<ITelegram> mTelegram;
    Status mStatus = Status::Success;
    std::unique_ptr<Impl> mImpl;
};

}  // namespace gwm
