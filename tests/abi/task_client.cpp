// A consumer of the IGWRBasicGpuTask binary interface, written the way a
// desktop client binds libgwmodelcuda: dlopen() the library, look up the
// extern "C" factories, and call the task through its vtable only.
//
//   task_client <libgwgpu.so> <input.bin> <mode: fit|predict|bulkfit|bulkpredict>
//
// The bulk modes move the data and the coefficients with the extern "C"
// GWRBasicGpuTask_SetData / _SetPredictLocations / _GetBetas helpers instead
// of the per-element virtual calls.
//
// input.bin: int32 n, p, geographic, adaptive, kernel, criterion(-1: no
// optimisation), n_pred; double bandwidth; then coords (n x 2 column-major),
// x (n x p column-major), y (n), prediction locations (n_pred x 2).
// Output (stdout, after the task's own telegram lines): "R ok <0|1>", then
// "R "-prefixed lines with the bandwidth, diagnostics and betas.
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/IGWRBasicGpuTask.h"

typedef IGWRBasicGpuTask* (*FitCreate)(int, int, int);
typedef IGWRBasicGpuTask* (*PredictCreate)(int, int, int, int);
typedef void (*Del)(IGWRBasicGpuTask*);
typedef int (*SetData)(IGWRBasicGpuTask*, const double*, const double*, const double*);
typedef int (*SetLoc)(IGWRBasicGpuTask*, const double*);
typedef int (*GetMat)(IGWRBasicGpuTask*, double*);

int main(int argc, char** argv)
{
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s lib input mode\n", argv[0]);
        return 2;
    }
    void* h = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        std::fprintf(stderr, "dlopen: %s\n", dlerror());
        return 2;
    }
    auto fitCreate = (FitCreate)dlsym(h, "GWRBasicGpuTaskFit_Create");
    auto predCreate = (PredictCreate)dlsym(h, "GWRBasicGpuTaskPredict_Create");
    auto del = (Del)dlsym(h, "GWRBasicGpuTask_Del");
    auto setData = (SetData)dlsym(h, "GWRBasicGpuTask_SetData");
    auto setLoc = (SetLoc)dlsym(h, "GWRBasicGpuTask_SetPredictLocations");
    auto getBetas = (GetMat)dlsym(h, "GWRBasicGpuTask_GetBetas");
    if (!fitCreate || !predCreate || !del || !setData || !setLoc || !getBetas) {
        std::fprintf(stderr, "missing factory\n");
        return 2;
    }
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 2;
    int hdr[7];
    double bw;
    if (std::fread(hdr, sizeof(int), 7, f) != 7 || std::fread(&bw, sizeof(double), 1, f) != 1) return 2;
    const int n = hdr[0], p = hdr[1], geo = hdr[2], adaptive = hdr[3], kernel = hdr[4], crit = hdr[5], nr = hdr[6];
    std::vector<double> coords(2 * (size_t)n), x((size_t)n * p), y(n), loc(2 * (size_t)nr);
    if (std::fread(coords.data(), sizeof(double), coords.size(), f) != coords.size() ||
        std::fread(x.data(), sizeof(double), x.size(), f) != x.size() ||
        std::fread(y.data(), sizeof(double), y.size(), f) != y.size() ||
        std::fread(loc.data(), sizeof(double), loc.size(), f) != loc.size())
        return 2;
    std::fclose(f);
    const bool bulk = argv[3][0] == 'b';
    const bool predict = argv[3][bulk ? 4 : 0] == 'p';
    IGWRBasicGpuTask* t = predict ? predCreate(n, p, 0, nr) : fitCreate(n, p, 0);
    if (bulk) {
        if (setData(t, x.data(), y.data(), coords.data()) != 0) return 3;
        if (predict && setLoc(t, loc.data()) != 0) return 3;
    } else {
        for (int i = 0; i < n; i++) {
            t->setY(i, y[i]);
            for (int k = 0; k < p; k++) t->setX(i, k, x[(size_t)i + (size_t)k * n]);
            t->setCoords(i, 0, coords[i]);  // (row, column, value), as the reference's quirk wants
            t->setCoords(i, 1, coords[(size_t)n + i]);
        }
        for (int i = 0; predict && i < nr; i++) {  // a fit task holds no prediction locations
            t->setPredictLocations(i, 0, loc[i]);
            t->setPredictLocations(i, 1, loc[(size_t)nr + i]);
        }
    }
    t->setCRSDistanceGergraphic(geo != 0);
    t->setBandwidthSize(bw);
    t->setBandwidthAdaptive(adaptive != 0);
    t->setBandwidthKernel(kernel);
    if (crit >= 0) t->enableBandwidthOptimization(crit);
    const bool ok = predict ? t->predict(true) : t->fit(true);
    std::fflush(stdout);
    std::printf("R ok %d\n", ok ? 1 : 0);
    if (ok) {
        const int rows = predict ? nr : n;
        if (!predict) {
            std::printf("R bandwidth %.17g\n", crit >= 0 ? t->optimizedBandwidth() : bw);
            std::printf("R aicc %.17g\nR rss %.17g\nR shat %.17g %.17g\n", t->diagnosticAICc(), t->diagnosticRSS(),
                        t->shat1(), t->shat2());
        }
        std::vector<double> b((size_t)rows * p);
        if (bulk && getBetas(t, b.data()) != 0) return 3;
        for (int i = 0; i < rows; i++) {
            std::printf("R");
            for (int k = 0; k < p; k++) std::printf(" %.17g", bulk ? b[(size_t)i + (size_t)k * rows] : t->betas(i, k));
            std::printf("\n");
        }
    }
    del(t);
    dlclose(h);
    return 0;
}
