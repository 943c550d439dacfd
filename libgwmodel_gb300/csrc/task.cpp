// task.cpp -- IGWRBasicGpuTask implementation over gwm::GWRBasic
// (libgwmodel src/gwmodelcuda/GWRBasicGpuTask.cpp:10-66 and
// include/gwmodelcuda/GWRBasicGpuTask.h:11-251 describe the behaviour).
#include <cstring>
#include "../../include/IGWRBasicGpuTask.h"

#include <exception>
#include <iostream>
#include <memory>
#include <vector>

#include "../../include/gwmodel_gb300/GWRBasic.h"

namespace {

// StdTelegram (src/gwmodelcuda/StdTelegram.cpp:6-24): messages to stdout.
class StdTelegram : public gwm::Logger {
public:
    void print(std::string message, LogLevel, std::string, std::string) override { std::cout << message + "\n"; }
};

constexpr int kCRSDistance = 0;  // Distance::DistanceType::CRSDistance (Distance.h:50-57)

class GWRBasicGpuTask final : public IGWRBasicGpuTask {
public:
    GWRBasicGpuTask(int nDp, int nVar, int distanceType, int nPredict = 0)
        : mX(nDp, nVar), mY(nDp, 1), mCoords(nDp, 2), mPredictLocations(nPredict, 2), mDistanceType(distanceType)
    {
    }

    void setX(int i, int k, double value) override { mX(i, k) = value; }
    void setY(int i, double value) override { mY(i, 0) = value; }
    void setCoords(int i, double u, double v) override { mCoords(i, (std::size_t)u) = v; }
    void setPredictLocations(int i, double u, double v) override { mPredictLocations(i, (std::size_t)u) = v; }

    void setDistanceType(int type) override { mDistanceType = type; }
    void setCRSDistanceGergraphic(bool isGeographic) override { mGeographic = isGeographic; }
    void setMinkwoskiDistancePoly(int poly) override { mPoly = poly; }
    void setMinkwoskiDistanceTheta(double theta) override { mTheta = theta; }

    void setBandwidthSize(double bw) override { mWeight.setBandwidth(bw); }
    void setBandwidthAdaptive(bool adaptive) override { mWeight.setAdaptive(adaptive); }
    void setBandwidthKernel(int kernel) override
    {
        mWeight.setKernel((gwm::BandwidthWeight::KernelFunctionType)kernel);
    }

    void enableBandwidthOptimization(int criterion) override
    {
        mIsOptimizeBandwidth = true;
        mCriterion = (gwm::GWRBasic::BandwidthSelectionCriterionType)criterion;
    }
    void enableVariablesOptimization(double threshold) override
    {
        mIsOptimizeVariables = true;
        mThreshold = threshold;
    }

    double betas(int i, int k) override { return mBetas(i, k); }
    double betasSE(int i, int k) override { return mBetasSE(i, k); }
    double shat1() override { return mSHat(0); }
    double shat2() override { return mSHat(1); }
    double qDiag(int i) override { return mQDiag(i); }
    unsigned long long sRows() override { return mS.n_rows; }
    double s(int i, int k) override { return mS(i, k); }

    double diagnosticRSS() override { return mDiagnostic.RSS; }
    double diagnosticAIC() override { return mDiagnostic.AIC; }
    double diagnosticAICc() override { return mDiagnostic.AICc; }
    double diagnosticENP() override { return mDiagnostic.ENP; }
    double diagnosticEDF() override { return mDiagnostic.EDF; }
    double diagnosticRSquare() override { return mDiagnostic.RSquare; }
    double diagnosticRSquareAdjust() override { return mDiagnostic.RSquareAdjust; }

    double optimizedBandwidth() override { return mOptimizedBandwidth; }
    unsigned long long selectedVarSize() override { return mSelectedVars.size(); }
    unsigned long long selectedVar(unsigned long long i) override { return mSelectedVars[i]; }
    unsigned long long variableSelectionCriterionSize() override { return mVarCriterion.size(); }
    unsigned long long variableSelectionCriterionItemVarSize(unsigned long long i) override
    {
        return mVarCriterion[i].first.size();
    }
    unsigned long long variableSelectionCriterionItemVar(unsigned long long i, unsigned long long j) override
    {
        return mVarCriterion[i].first[j];
    }
    double variableSelectionCriterionItemValue(unsigned long long i) override { return mVarCriterion[i].second; }

    // GWRBasicGpuTask::fit (GWRBasicGpuTask.cpp:10-47): any exception -> false.
    bool fit(bool hasIntercept) override
    {
        if (mDistanceType != kCRSDistance) return false;  // only CRS distances run on this engine
        try {
            gwm::CRSDistance d(mGeographic);
            gwm::SpatialWeight sw(&mWeight, &d);
            gwm::GWRBasic algorithm(mX, mY, mCoords, sw, true, hasIntercept);
            algorithm.setIsAutoselectBandwidth(mIsOptimizeBandwidth);
            algorithm.setBandwidthSelectionCriterion(mCriterion);
            algorithm.setIsAutoselectIndepVars(mIsOptimizeVariables);
            algorithm.setIndepVarSelectionThreshold(mThreshold);
            algorithm.setParallelType(gwm::ParallelType::CUDA);
            algorithm.setTelegram(std::unique_ptr<gwm::ITelegram>(new StdTelegram()));
            algorithm.fit();
            mBetas = algorithm.betas();
            mBetasSE = algorithm.betasSE();
            mSHat = algorithm.sHat();
            mQDiag = algorithm.qDiag();
            mS = algorithm.s();
            mDiagnostic = algorithm.diagnostic();
            if (mIsOptimizeBandwidth) mOptimizedBandwidth = algorithm.spatialWeight().weight()->bandwidth();
            if (mIsOptimizeVariables) {
                mSelectedVars = algorithm.selectedVariables();
                mVarCriterion = algorithm.indepVarsSelectionCriterionList();
            }
        } catch (const std::exception&) {
            return false;
        }
        return true;
    }

    // GWRBasicGpuTask::predict (GWRBasicGpuTask.cpp:49-66): any exception -> false.
    bool predict(bool hasIntercept) override
    {
        if (mDistanceType != kCRSDistance) return false;
        try {
            gwm::CRSDistance d(mGeographic);
            gwm::SpatialWeight sw(&mWeight, &d);
            gwm::GWRBasic algorithm(mX, mY, mCoords, sw, true, hasIntercept);
            algorithm.setParallelType(gwm::ParallelType::CUDA);
            algorithm.setTelegram(std::unique_ptr<gwm::ITelegram>(new StdTelegram()));
            algorithm.predict(mPredictLocations);
            mBetas = algorithm.betas();
        } catch (const std::exception&) {
            return false;
        }
        return true;
    }

    // bulk I/O (the extern "C" GWRBasicGpuTask_* helpers)
    void setData(const double* x, const double* y, const double* coords)
    {
        std::memcpy(mX.memptr(), x, sizeof(double) * mX.n_elem());
        std::memcpy(mY.memptr(), y, sizeof(double) * mY.n_elem());
        std::memcpy(mCoords.memptr(), coords, sizeof(double) * mCoords.n_elem());
    }
    void setPredictLocations(const double* locations)
    {
        std::memcpy(mPredictLocations.memptr(), locations, sizeof(double) * mPredictLocations.n_elem());
    }
    const gwm::mat& betasMatrix() const { return mBetas; }
    const gwm::mat& betasSEMatrix() const { return mBetasSE; }

private:
    gwm::mat mX, mY, mCoords, mPredictLocations;
    gwm::mat mBetas, mBetasSE, mSHat, mQDiag, mS;
    int mDistanceType = kCRSDistance;
    bool mGeographic = false;
    int mPoly = 2;
    double mTheta = 0.0;
    gwm::BandwidthWeight mWeight;
    bool mIsOptimizeBandwidth = false;
    gwm::GWRBasic::BandwidthSelectionCriterionType mCriterion = gwm::GWRBasic::CV;  // GWRBasicGpuTask.h:28
    bool mIsOptimizeVariables = false;
    double mThreshold = 3.0;
    gwm::RegressionDiagnostic mDiagnostic{};
    double mOptimizedBandwidth = 0.0;
    std::vector<std::size_t> mSelectedVars;
    gwm::VariablesCriterionList mVarCriterion;
};

}  // namespace

extern "C" int GWRBasicGpuTask_SetData(IGWRBasicGpuTask* task, const double* x, const double* y, const double* coords)
{
    auto* t = dynamic_cast<GWRBasicGpuTask*>(task);
    if (!t || !x || !y || !coords) return -1;
    t->setData(x, y, coords);
    return 0;
}

extern "C" int GWRBasicGpuTask_SetPredictLocations(IGWRBasicGpuTask* task, const double* locations)
{
    auto* t = dynamic_cast<GWRBasicGpuTask*>(task);
    if (!t || !locations) return -1;
    t->setPredictLocations(locations);
    return 0;
}

extern "C" int GWRBasicGpuTask_GetBetas(IGWRBasicGpuTask* task, double* out)
{
    auto* t = dynamic_cast<GWRBasicGpuTask*>(task);
    if (!t || !out) return -1;
    const gwm::mat& m = t->betasMatrix();
    if (m.n_elem()) std::memcpy(out, m.memptr(), sizeof(double) * m.n_elem());
    return 0;
}

extern "C" int GWRBasicGpuTask_GetBetasSE(IGWRBasicGpuTask* task, double* out)
{
    auto* t = dynamic_cast<GWRBasicGpuTask*>(task);
    if (!t || !out) return -1;
    const gwm::mat& m = t->betasSEMatrix();
    if (m.n_elem()) std::memcpy(out, m.memptr(), sizeof(double) * m.n_elem());
    return 0;
}

extern "C" IGWRBasicGpuTask* GWRBasicGpuTaskFit_Create(int nDp, int nVar, int distanceType)
{
    try {
        return new GWRBasicGpuTask(nDp, nVar, distanceType);
    } catch (...) {
        return nullptr;
    }
}

extern "C" IGWRBasicGpuTask* GWRBasicGpuTaskPredict_Create(int nDp, int nVar, int distanceType, int nPredictPoints)
{
    try {
        return new GWRBasicGpuTask(nDp, nVar, distanceType, nPredictPoints);
    } catch (...) {
        return nullptr;
    }
}

// The interface has no virtual destructor (as in the reference), so delete
// through the concrete type.
extern "C" void GWRBasicGpuTask_Del(IGWRBasicGpuTask* pInstance)
{
    delete static_cast<GWRBasicGpuTask*>(pInstance);
}
