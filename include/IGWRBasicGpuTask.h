/*
 * IGWRBasicGpuTask.h -- binary drop-in for libgwmodelcuda's task interface.
 *
 * Replaces include/gwmodelcuda/IGWRBasicGpuTask.h:14-65 of libgwmodel: the
 * virtual methods are declared in the same order, so an application compiled
 * against the reference header (e.g. a desktop client that dlopen()s the
 * library and calls the three factories) gets the same vtable layout from
 * libgwgpu.so.  The implementation runs GWRBasic on the GB300 engine.
 *
 * Preserved quirk (GWRBasicGpuTask.h:138-141 of the reference): setCoords(i,
 * u, v) stores v at row i, column (int)u -- callers pass (row, column, value).
 */
#ifndef GWGPU_IGWRBASICGPUTASK_H
#define GWGPU_IGWRBASICGPUTASK_H

#if defined(_WIN32)
#define GWMODELCUDA_API __declspec(dllexport)
#else
#define GWMODELCUDA_API __attribute__((visibility("default")))
#endif

class GWMODELCUDA_API IGWRBasicGpuTask
{
public:
    virtual void setX(int i, int k, double value) = 0;
    virtual void setY(int i, double value) = 0;
    virtual void setCoords(int i, double u, double v) = 0;
    virtual void setPredictLocations(int i, double u, double v) = 0;

    virtual void setDistanceType(int type) = 0;
    virtual void setCRSDistanceGergraphic(bool isGeographic) = 0;
    virtual void setMinkwoskiDistancePoly(int poly) = 0;
    virtual void setMinkwoskiDistanceTheta(double theta) = 0;

    virtual void setBandwidthSize(double bw) = 0;
    virtual void setBandwidthAdaptive(bool adaptive) = 0;
    virtual void setBandwidthKernel(int kernel) = 0;

    virtual void enableBandwidthOptimization(int criterion) = 0;
    virtual void enableVariablesOptimization(double threshold) = 0;

    virtual double betas(int i, int k) = 0;
    virtual double betasSE(int i, int k) = 0;
    virtual double shat1() = 0;
    virtual double shat2() = 0;
    virtual double qDiag(int i) = 0;
    virtual unsigned long long sRows() = 0;
    virtual double s(int i, int k) = 0;

    virtual double diagnosticRSS() = 0;
    virtual double diagnosticAIC() = 0;
    virtual double diagnosticAICc() = 0;
    virtual double diagnosticENP() = 0;
    virtual double diagnosticEDF() = 0;
    virtual double diagnosticRSquare() = 0;
    virtual double diagnosticRSquareAdjust() = 0;

    virtual double optimizedBandwidth() = 0;
    virtual unsigned long long selectedVarSize() = 0;
    virtual unsigned long long selectedVar(unsigned long long i) = 0;
    virtual unsigned long long variableSelectionCriterionSize() = 0;
    virtual unsigned long long variableSelectionCriterionItemVarSize(unsigned long long i) = 0;
    virtual unsigned long long variableSelectionCriterionItemVar(unsigned long long i, unsigned long long j) = 0;
    virtual double variableSelectionCriterionItemValue(unsigned long long i) = 0;

    virtual bool fit(bool hasIntercept) = 0;

    virtual bool predict(bool hasIntercept) = 0;
};

extern "C" GWMODELCUDA_API IGWRBasicGpuTask* GWRBasicGpuTaskFit_Create(int nDp, int nVar, int distanceType);
extern "C" GWMODELCUDA_API IGWRBasicGpuTask* GWRBasicGpuTaskPredict_Create(int nDp, int nVar, int distanceType,
                                                                           int nPredictPoints);
extern "C" GWMODELCUDA_API void GWRBasicGpuTask_Del(IGWRBasicGpuTask* pInstance);

/* Bulk I/O beside the per-element vtable calls (setX/setY/setCoords and the
 * betas(i, k) getters cost one virtual call per element,
 * GWRBasicGpuTask.h:128-146 of the reference).  They are plain functions, so
 * the interface's vtable is unchanged; each returns 0, or -1 when the task is
 * not one of this library's or a pointer is null.  Matrices are column-major:
 * x nDp x nVar, coords nDp x 2, locations nPredictPoints x 2; the getters
 * write rows x nVar where rows is nDp after fit() and nPredictPoints after
 * predict(). */
extern "C" GWMODELCUDA_API int GWRBasicGpuTask_SetData(IGWRBasicGpuTask* task, const double* x, const double* y,
                                                       const double* coords);
extern "C" GWMODELCUDA_API int GWRBasicGpuTask_SetPredictLocations(IGWRBasicGpuTask* task, const double* locations);
extern "C" GWMODELCUDA_API int GWRBasicGpuTask_GetBetas(IGWRBasicGpuTask* task, double* out);
extern "C" GWMODELCUDA_API int GWRBasicGpuTask_GetBetasSE(IGWRBasicGpuTask* task, double* out);

#endif /* GWGPU_IGWRBASICGPUTASK_H */
