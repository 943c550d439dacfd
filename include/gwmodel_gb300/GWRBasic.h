// GWRBasic.h -- C++ drop-in for gwm::GWRBasic backed by the GB300 engine.
//
// Same setters, fit() and getters as libgwmodel's GWRBasic
// (include/gwmodelpp/GWRBasic.h:29-757, GWRBase.h:41-184,
// SpatialAlgorithm.h:91, SpatialMonoscaleAlgorithm.h:93, Algorithm.h:122-217)
// and the same tagged telegram messages.  Armadillo is not required: matrices
// are the small column-major gwm::mat below (element (i, j) at i + j*n_rows,
// Armadillo's layout), so callers that hold an arma::mat pass its memptr().
// Every fit runs on the GPU, whatever ParallelType says; there is no CPU path.
#pragma once

#include <cfloat>
#include <cstddef>
#include <memory>
#include <optional>
#include <string>
#include <utility>
#include <vector>

namespace gwm {

// ParallelType (IParallelizable.h:15-20).
enum ParallelType { SerialOnly = 1 << 0, OpenMP = 1 << 1, CUDA = 1 << 2 };

// Status (Status.h:10-14).
enum class Status { Success = 0, Terminated };

// RegressionDiagnostic (RegressionDiagnostic.h:11-20).
struct RegressionDiagnostic {
    double RSS, AIC, AICc, ENP, EDF, RSquare, RSquareAdjust;
};

// ITelegram / Logger (Logger.h:31-83).
struct ITelegram {
    enum class LogLevel { LOG_EMERG = 0, LOG_ALERT, LOG_CRIT, LOG_ERR, LOG_WARNING, LOG_NOTICE, LOG_INFO, LOG_DEBUG };
    virtual ~ITelegram() {}
    virtual void print(std::string message, LogLevel level, std::string fun_name, std::string file_name) = 0;
    virtual void progress(std::size_t current, std::size_t total, std::string fun_name, std::string file_name) = 0;
    virtual void progress(double percent, std::string fun_name, std::string file_name) = 0;
    virtual bool stop() = 0;
};

class Logger : public ITelegram {
public:
    void print(std::string, LogLevel, std::string, std::string) override {}
    void progress(std::size_t, std::size_t, std::string, std::string) override {}
    void progress(double, std::string, std::string) override {}
    bool stop() override { return false; }
};

// Minimal column-major matrix (a vector is n x 1).
class mat {
public:
    mat() = default;
    mat(std::size_t rows, std::size_t cols, double fill = 0.0) : n_rows(rows), n_cols(cols), data_(rows * cols, fill) {}
    mat(std::size_t rows, std::size_t cols, const double* colmajor)
        : n_rows(rows), n_cols(cols), data_(colmajor, colmajor + rows * cols) {}
    double& operator()(std::size_t i, std::size_t j) { return data_[i + j * n_rows]; }
    double operator()(std::size_t i, std::size_t j = 0) const { return data_[i + j * n_rows]; }
    double* memptr() { return data_.data(); }
    const double* memptr() const { return data_.data(); }
    std::size_t n_elem() const { return data_.size(); }
    std::size_t n_rows = 0, n_cols = 0;

private:
    std::vector<double> data_;
};
using vec = mat;

// CRSDistance (spatialweight/CRSDistance.h): planar or geographic.
class CRSDistance {
public:
    CRSDistance() = default;
    explicit CRSDistance(bool isGeographic) : mGeographic(isGeographic) {}
    bool geographic() const { return mGeographic; }
    void setGeographic(bool g) { mGeographic = g; }

private:
    bool mGeographic = false;
};

// BandwidthWeight (spatialweight/BandwidthWeight.h:46-53, 68-121).
class BandwidthWeight {
public:
    enum KernelFunctionType { Gaussian, Exponential, Bisquare, Tricube, Boxcar };
    BandwidthWeight() = default;
    BandwidthWeight(double size, bool adaptive, KernelFunctionType kernel)
        : mBandwidth(size), mAdaptive(adaptive), mKernel(kernel) {}
    double bandwidth() const { return mBandwidth; }
    void setBandwidth(double v) { mBandwidth = v; }
    bool adaptive() const { return mAdaptive; }
    void setAdaptive(bool v) { mAdaptive = v; }
    KernelFunctionType kernel() const { return mKernel; }
    void setKernel(KernelFunctionType k) { mKernel = k; }

private:
    double mBandwidth = 0.0;
    bool mAdaptive = true;
    KernelFunctionType mKernel = Gaussian;
};

// SpatialWeight (spatialweight/SpatialWeight.h:72-111): deep copies of both parts.
class SpatialWeight {
public:
    SpatialWeight() = default;
    SpatialWeight(const BandwidthWeight* weight, const CRSDistance* distance) : mWeight(*weight), mDistance(*distance) {}
    template <class T = BandwidthWeight>
    const BandwidthWeight* weight() const { return &mWeight; }
    BandwidthWeight* weightMutable() { return &mWeight; }
    const CRSDistance* distance() const { return &mDistance; }
    void setWeight(const BandwidthWeight& w) { mWeight = w; }

private:
    BandwidthWeight mWeight;
    CRSDistance mDistance;
};

using BandwidthCriterionList = std::vector<std::pair<double, double>>;
using VariablesCriterionList = std::vector<std::pair<std::vector<std::size_t>, double>>;

// Numeric form of the engine: the FP64 drop-in, or tensor-core mixed precision.
enum class Precision { FP64 = 0, Mixed = 1 };

class GWRBasic {
public:
    enum BandwidthSelectionCriterionType { AIC, CV };

    GWRBasic();
    GWRBasic(const mat& x, const vec& y, const mat& coords, const SpatialWeight& spatialWeight,
             bool hasHatMatrix = true, bool hasIntercept = true);
    ~GWRBasic();
    GWRBasic(const GWRBasic&) = delete;
    GWRBasic& operator=(const GWRBasic&) = delete;

    // SpatialAlgorithm / GWRBase / SpatialMonoscaleAlgorithm setters
    void setCoords(const mat& coords) { mCoords = coords; }
    const mat& coords() const { return mCoords; }
    void setDependentVariable(const vec& y) { mY = y; }
    const vec& dependentVariable() const { return mY; }
    void setIndependentVariables(const mat& x) { mX = x; }
    const mat& independentVariables() const { return mX; }
    void setSpatialWeight(const SpatialWeight& sw) { mSpatialWeight = sw; }
    const SpatialWeight& spatialWeight() const { return mSpatialWeight; }
    bool hasIntercept() const { return mHasIntercept; }
    void setHasIntercept(bool has) { mHasIntercept = has; }

    // GWRBasic setters (GWRBasic.h:145-310, 685-690)
    bool isAutoselectBandwidth() const { return mIsAutoselectBandwidth; }
    void setIsAutoselectBandwidth(bool v) { mIsAutoselectBandwidth = v; }
    BandwidthSelectionCriterionType bandwidthSelectionCriterion() const { return mBandwidthSelectionCriterion; }
    void setBandwidthSelectionCriterion(const BandwidthSelectionCriterionType& criterion);
    void setGoldenUpperBounds(double value) { mGoldenUpperBounds = value; }
    void setGoldenLowerBounds(double value) { mGoldenLowerBounds = value; }
    bool isAutoselectIndepVars() const { return mIsAutoselectIndepVars; }
    void setIsAutoselectIndepVars(bool v) { mIsAutoselectIndepVars = v; }
    double indepVarSelectionThreshold() const { return mIndepVarSelectionThreshold; }
    void setIndepVarSelectionThreshold(double t) { mIndepVarSelectionThreshold = t; }
    bool hasHatMatrix() const { return mHasHatMatrix; }
    void setHasHatMatrix(bool has) { mHasHatMatrix = has; }
    int parallelAbility() const { return SerialOnly | OpenMP | CUDA; }
    ParallelType parallelType() const { return mParallelType; }
    void setParallelType(const ParallelType& type);
    void setOmpThreadNum(int threadNum) { mOmpThreadNum = threadNum; }
    void setGPUId(int gpuId) { mGpuId = gpuId; }
    void setGroupSize(std::size_t size) { mGroupLength = size; }
    void setPrecision(Precision p) { mPrecision = p; }
    Precision precision() const { return mPrecision; }

    // Algorithm (Algorithm.h:122-217)
    void setTelegram(std::unique_ptr<ITelegram> telegram) { mTelegram = std::move(telegram); }
    const std::unique_ptr<ITelegram>& telegram() const { return mTelegram; }
    Status status() const { return mStatus; }
    bool isValid();

    mat fit();
    // GWRBasic::predict (GWRBasic.cpp:130-155): coefficients at the given
    // locations (rows of a nRp x 2 matrix) at the spatial weight's bandwidth.
    mat predict(const mat& locations);

    // results
    const mat& betas() const { return mBetas; }
    const mat& betasSE() const { return mBetasSE; }
    const vec& sHat() const { return mSHat; }
    const vec& qDiag() const { return mQDiag; }
    const mat& s() const { return mS; }
    RegressionDiagnostic diagnostic() const { return mDiagnostic; }
    const BandwidthCriterionList& bandwidthSelectionCriterionList() const { return mBandwidthSelectionCriterionList; }
    const VariablesCriterionList& indepVarsSelectionCriterionList() const { return mIndepVarsSelectionCriterionList; }
    std::vector<std::size_t> selectedVariables() const { return mSelectedIndepVars; }

private:
    struct Impl;
    double bandwidthCriterion(const BandwidthWeight& w);
    double indepVarsCriterion(const std::vector<std::size_t>& vars);

    mat mX, mCoords, mBetas, mBetasSE, mS;
    vec mY, mSHat, mQDiag;
    SpatialWeight mSpatialWeight;
    bool mHasIntercept = true, mHasHatMatrix = true;
    bool mIsAutoselectBandwidth = false, mIsAutoselectIndepVars = false;
    double mIndepVarSelectionThreshold = 3.0;
    BandwidthSelectionCriterionType mBandwidthSelectionCriterion = AIC;
    // the reference's criterion function pointer starts at CV (GWRBasic.h:739)
    BandwidthSelectionCriterionType mCriterionFunction = CV;
    std::optional<double> mGoldenUpperBounds, mGoldenLowerBounds;
    ParallelType mParallelType = SerialOnly;
    int mOmpThreadNum = 8, mGpuId = 0;
    std::size_t mGroupLength = 64;
    Precision mPrecision = Precision::FP64;
    double mBandwidthLastCriterion = DBL_MAX;
    std::size_t mIndepVarSelectionProgressTotal = 0, mIndepVarSelectionProgressCurrent = 0;
    BandwidthCriterionList mBandwidthSelectionCriterionList;
    VariablesCriterionList mIndepVarsSelectionCriterionList;
    std::vector<std::size_t> mSelectedIndepVars;
    RegressionDiagnostic mDiagnostic{};
    std::unique_ptr<ITelegram> mTelegram;
    Status mStatus = Status::Success;
    std::unique_ptr<Impl> mImpl;
};

}  // namespace gwm
