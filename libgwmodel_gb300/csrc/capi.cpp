// capi.cpp -- extern "C" layer of include/gwgpu.h over gwm::GWRBasic and the engine.
#include "../../include/gwgpu.h"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/gwmodel_gb300/GWRBasic.h"
#include "../../include/gwmodel_gb300/GWRMultiscale.h"
#include "engine.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* msg)
{
    g_last_error = msg ? msg : "";
    return code;
}

template <class F>
int guarded(F&& f)
{
    try {
        f();
        return GWGPU_OK;
    } catch (const gwgpu::NotSPDError& e) {
        return fail(GWGPU_ERR_NOT_SPD, e.what());
    } catch (const gwgpu::CudaError& e) {
        return fail(GWGPU_ERR_CUDA, e.what());
    } catch (const std::out_of_range& e) {
        return fail(GWGPU_ERR_RANGE, e.what());
    } catch (const std::invalid_argument& e) {
        return fail(GWGPU_ERR_INVALID, e.what());
    } catch (const std::logic_error& e) {
        return fail(GWGPU_ERR_INVALID, e.what());
    } catch (const std::bad_alloc&) {
        return fail(GWGPU_ERR_RUNTIME, "out of host memory");
    } catch (const std::exception& e) {
        return fail(GWGPU_ERR_RUNTIME, e.what());
    }
}

// ITelegram over the C callbacks.
class CTelegram : public gwm::ITelegram {
public:
    explicit CTelegram(const gwgpu_telegram& t) : t_(t) {}
    void print(std::string message, LogLevel level, std::string fun, std::string file) override
    {
        if (t_.print) t_.print(t_.user, message.c_str(), (int)level, fun.c_str(), file.c_str());
    }
    void progress(std::size_t current, std::size_t total, std::string fun, std::string file) override
    {
        if (t_.progress) t_.progress(t_.user, current, total, fun.c_str(), file.c_str());
    }
    void progress(double percent, std::string fun, std::string file) override
    {
        if (t_.progress_percent) t_.progress_percent(t_.user, percent, fun.c_str(), file.c_str());
    }
    bool stop() override { return t_.stop ? t_.stop(t_.user) != 0 : false; }

private:
    gwgpu_telegram t_;
};

}  // namespace

namespace gwgpu {
// Sets the calling thread's gwgpu_last_error() message (used by entry points
// defined in other translation units).
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }
}  // namespace gwgpu

struct gwgpu_gwr {
    gwm::GWRBasic alg;
    double bandwidth = 0.0;
    bool adaptive = true;
    int kernel = GWGPU_GAUSSIAN;
    bool geographic = false;
};

struct gwgpu_mgwr {
    gwm::GWRMultiscale alg;
};

struct gwgpu_engine {
    explicit gwgpu_engine(int device) : eng(device) {}
    gwgpu::Engine eng;
};

extern "C" {

int gwgpu_version(void) { return 10000; }

const char* gwgpu_last_error(void) { return g_last_error.c_str(); }

int gwgpu_device_count(int* count)
{
    if (!count) return fail(GWGPU_ERR_INVALID, "null pointer");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        return fail(GWGPU_ERR_CUDA, cudaGetErrorString(e));
    }
    return GWGPU_OK;
}

// ------------------------------------------------------------------- gwr

int gwgpu_gwr_create(gwgpu_gwr** out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null pointer");
    return guarded([&] { *out = new gwgpu_gwr(); });
}

void gwgpu_gwr_destroy(gwgpu_gwr* g) { delete g; }

#define GWR_CHECK(g) \
    if (!(g)) return fail(GWGPU_ERR_INVALID, "null handle")

int gwgpu_gwr_set_coords(gwgpu_gwr* g, int n, const double* coords)
{
    GWR_CHECK(g);
    if (n < 0 || (!coords && n)) return fail(GWGPU_ERR_INVALID, "bad coords");
    return guarded([&] { g->alg.setCoords(gwm::mat(n, 2, coords)); });
}

int gwgpu_gwr_set_dependent_variable(gwgpu_gwr* g, int n, const double* y)
{
    GWR_CHECK(g);
    if (n < 0 || (!y && n)) return fail(GWGPU_ERR_INVALID, "bad y");
    return guarded([&] { g->alg.setDependentVariable(gwm::vec(n, 1, y)); });
}

int gwgpu_gwr_set_independent_variables(gwgpu_gwr* g, int n, int p, const double* x)
{
    GWR_CHECK(g);
    if (n < 0 || p < 0 || (!x && n && p)) return fail(GWGPU_ERR_INVALID, "bad x");
    return guarded([&] { g->alg.setIndependentVariables(gwm::mat(n, p, x)); });
}

int gwgpu_gwr_set_spatial_weight(gwgpu_gwr* g, double bandwidth, int adaptive, int kernel, int geographic)
{
    GWR_CHECK(g);
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    gwm::BandwidthWeight w(bandwidth, adaptive != 0, (gwm::BandwidthWeight::KernelFunctionType)kernel);
    gwm::CRSDistance d(geographic != 0);
    g->alg.setSpatialWeight(gwm::SpatialWeight(&w, &d));
    return GWGPU_OK;
}

int gwgpu_gwr_set_is_autoselect_bandwidth(gwgpu_gwr* g, int on)
{
    GWR_CHECK(g);
    g->alg.setIsAutoselectBandwidth(on != 0);
    return GWGPU_OK;
}

int gwgpu_gwr_set_bandwidth_selection_criterion(gwgpu_gwr* g, int criterion)
{
    GWR_CHECK(g);
    if (criterion != GWGPU_AIC && criterion != GWGPU_CV) return fail(GWGPU_ERR_INVALID, "unknown criterion");
    g->alg.setBandwidthSelectionCriterion((gwm::GWRBasic::BandwidthSelectionCriterionType)criterion);
    return GWGPU_OK;
}

int gwgpu_gwr_set_golden_upper_bounds(gwgpu_gwr* g, double value)
{
    GWR_CHECK(g);
    g->alg.setGoldenUpperBounds(value);
    return GWGPU_OK;
}

int gwgpu_gwr_set_golden_lower_bounds(gwgpu_gwr* g, double value)
{
    GWR_CHECK(g);
    g->alg.setGoldenLowerBounds(value);
    return GWGPU_OK;
}

int gwgpu_gwr_set_has_hat_matrix(gwgpu_gwr* g, int on)
{
    GWR_CHECK(g);
    g->alg.setHasHatMatrix(on != 0);
    return GWGPU_OK;
}

int gwgpu_gwr_set_has_intercept(gwgpu_gwr* g, int on)
{
    GWR_CHECK(g);
    g->alg.setHasIntercept(on != 0);
    return GWGPU_OK;
}

int gwgpu_gwr_set_is_autoselect_indep_vars(gwgpu_gwr* g, int on)
{
    GWR_CHECK(g);
    g->alg.setIsAutoselectIndepVars(on != 0);
    return GWGPU_OK;
}

int gwgpu_gwr_set_indep_var_selection_threshold(gwgpu_gwr* g, double threshold)
{
    GWR_CHECK(g);
    g->alg.setIndepVarSelectionThreshold(threshold);
    return GWGPU_OK;
}

int gwgpu_gwr_set_parallel_type(gwgpu_gwr* g, int type)
{
    GWR_CHECK(g);
    g->alg.setParallelType((gwm::ParallelType)type);
    return GWGPU_OK;
}

int gwgpu_gwr_set_omp_thread_num(gwgpu_gwr* g, int threads)
{
    GWR_CHECK(g);
    g->alg.setOmpThreadNum(threads);
    return GWGPU_OK;
}

int gwgpu_gwr_set_gpu_id(gwgpu_gwr* g, int gpu)
{
    GWR_CHECK(g);
    g->alg.setGPUId(gpu);
    return GWGPU_OK;
}

int gwgpu_gwr_set_group_size(gwgpu_gwr* g, size_t size)
{
    GWR_CHECK(g);
    g->alg.setGroupSize(size);
    return GWGPU_OK;
}

int gwgpu_gwr_set_precision(gwgpu_gwr* g, int precision)
{
    GWR_CHECK(g);
    if (precision != GWGPU_FP64 && precision != GWGPU_MIXED) return fail(GWGPU_ERR_INVALID, "unknown precision");
    g->alg.setPrecision((gwm::Precision)precision);
    return GWGPU_OK;
}

int gwgpu_gwr_set_telegram(gwgpu_gwr* g, const gwgpu_telegram* t)
{
    GWR_CHECK(g);
    return guarded([&] {
        if (t)
            g->alg.setTelegram(std::unique_ptr<gwm::ITelegram>(new CTelegram(*t)));
        else
            g->alg.setTelegram(std::unique_ptr<gwm::ITelegram>(new gwm::Logger()));
    });
}

int gwgpu_gwr_fit(gwgpu_gwr* g)
{
    GWR_CHECK(g);
    return guarded([&] { g->alg.fit(); });
}

int gwgpu_gwr_predict(gwgpu_gwr* g, int nr, const double* locations, double* betas)
{
    GWR_CHECK(g);
    if (nr < 1 || !locations) return fail(GWGPU_ERR_INVALID, "need at least one prediction location");
    return guarded([&] {
        gwm::mat loc((std::size_t)nr, 2, locations);
        gwm::mat b = g->alg.predict(loc);
        if (betas) std::memcpy(betas, b.memptr(), sizeof(double) * b.n_elem());
    });
}

int gwgpu_gwr_status(gwgpu_gwr* g)
{
    if (!g) return -1;
    return (int)g->alg.status();
}

int gwgpu_gwr_shape(gwgpu_gwr* g, int* n, int* p, int* s_rows)
{
    GWR_CHECK(g);
    if (n) *n = (int)g->alg.betas().n_rows;
    if (p) *p = (int)g->alg.betas().n_cols;
    if (s_rows) *s_rows = (int)g->alg.s().n_rows;
    return GWGPU_OK;
}

static int copy_out(const gwm::mat& m, double* out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    if (m.n_elem()) std::memcpy(out, m.memptr(), sizeof(double) * m.n_elem());
    return GWGPU_OK;
}

int gwgpu_gwr_betas(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    return copy_out(g->alg.betas(), out);
}

int gwgpu_gwr_betas_se(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    return copy_out(g->alg.betasSE(), out);
}

int gwgpu_gwr_shat(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    return copy_out(g->alg.sHat(), out);
}

int gwgpu_gwr_qdiag(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    return copy_out(g->alg.qDiag(), out);
}

int gwgpu_gwr_s(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    return copy_out(g->alg.s(), out);
}

int gwgpu_gwr_diagnostic(gwgpu_gwr* g, double* out)
{
    GWR_CHECK(g);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    gwm::RegressionDiagnostic d = g->alg.diagnostic();
    out[0] = d.RSS;
    out[1] = d.AIC;
    out[2] = d.AICc;
    out[3] = d.ENP;
    out[4] = d.EDF;
    out[5] = d.RSquare;
    out[6] = d.RSquareAdjust;
    return GWGPU_OK;
}

int gwgpu_gwr_bandwidth(gwgpu_gwr* g, double* bandwidth)
{
    GWR_CHECK(g);
    if (!bandwidth) return fail(GWGPU_ERR_INVALID, "null output");
    *bandwidth = g->alg.spatialWeight().weight()->bandwidth();
    return GWGPU_OK;
}

int gwgpu_gwr_bandwidth_criterion_list(gwgpu_gwr* g, int* count, double* bw, double* value)
{
    GWR_CHECK(g);
    const auto& l = g->alg.bandwidthSelectionCriterionList();
    if (count) *count = (int)l.size();
    for (size_t i = 0; i < l.size(); i++) {
        if (bw) bw[i] = l[i].first;
        if (value) value[i] = l[i].second;
    }
    return GWGPU_OK;
}

int gwgpu_gwr_selected_vars(gwgpu_gwr* g, int* count, int* vars)
{
    GWR_CHECK(g);
    auto v = g->alg.selectedVariables();
    if (count) *count = (int)v.size();
    if (vars)
        for (size_t i = 0; i < v.size(); i++) vars[i] = (int)v[i];
    return GWGPU_OK;
}

int gwgpu_gwr_var_criterion_list(gwgpu_gwr* g, int* count, int* total_vars, int* lens, int* vars, double* value)
{
    GWR_CHECK(g);
    const auto& l = g->alg.indepVarsSelectionCriterionList();
    if (count) *count = (int)l.size();
    int off = 0;
    for (size_t i = 0; i < l.size(); i++) {
        if (lens) lens[i] = (int)l[i].first.size();
        if (value) value[i] = l[i].second;
        for (size_t k = 0; k < l[i].first.size(); k++) {
            if (vars) vars[off] = (int)l[i].first[k];
            off++;
        }
    }
    if (total_vars) *total_vars = off;
    return GWGPU_OK;
}

// ---------------------------------------------------------------- engine

int gwgpu_engine_create(int device, gwgpu_engine** out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null pointer");
    *out = nullptr;
    return guarded([&] { *out = new gwgpu_engine(device); });
}

void gwgpu_engine_destroy(gwgpu_engine* e) { delete e; }

#define ENG_CHECK(e) \
    if (!(e)) return fail(GWGPU_ERR_INVALID, "null handle")

int gwgpu_engine_set_data(gwgpu_engine* e, int n, int p, const double* x, const double* y, const double* coords,
                          int geographic)
{
    ENG_CHECK(e);
    if (!x || !y || !coords) return fail(GWGPU_ERR_INVALID, "null input");
    return guarded([&] { e->eng.setData(n, p, x, y, coords, geographic != 0); });
}

int gwgpu_engine_set_precision(gwgpu_engine* e, int precision)
{
    ENG_CHECK(e);
    if (precision != GWGPU_FP64 && precision != GWGPU_MIXED) return fail(GWGPU_ERR_INVALID, "unknown precision");
    e->eng.setPrecision(precision);
    return GWGPU_OK;
}

int gwgpu_engine_set_refinement(gwgpu_engine* e, int steps, int refine_search)
{
    ENG_CHECK(e);
    if (steps < 0 || steps > 8) return fail(GWGPU_ERR_INVALID, "refinement steps must be in [0, 8]");
    e->eng.setRefinement(steps, refine_search != 0);
    return GWGPU_OK;
}

int gwgpu_engine_set_flush_tiles(gwgpu_engine* e, int tiles)
{
    ENG_CHECK(e);
    if (tiles < 2 || tiles > 1 << 20) return fail(GWGPU_ERR_INVALID, "flush tiles must be in [2, 2^20]");
    e->eng.setFlushTiles(tiles);
    return GWGPU_OK;
}

int gwgpu_engine_set_tc_wait_limit(gwgpu_engine* e, unsigned polls)
{
    ENG_CHECK(e);
    e->eng.setTcWaitLimit(polls);
    return GWGPU_OK;
}

int gwgpu_engine_criterion(gwgpu_engine* e, double bandwidth, int adaptive, int kernel, int criterion, double* value)
{
    ENG_CHECK(e);
    if (!value) return fail(GWGPU_ERR_INVALID, "null output");
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    return guarded([&] { *value = e->eng.criterion(bandwidth, adaptive != 0, kernel, criterion); });
}

int gwgpu_engine_global_criterion(gwgpu_engine* e, int ncols, const int* cols, double* value)
{
    ENG_CHECK(e);
    if (!value || !cols) return fail(GWGPU_ERR_INVALID, "null pointer");
    return guarded([&] { *value = e->eng.globalCriterion(std::vector<int>(cols, cols + ncols)); });
}

int gwgpu_engine_fit(gwgpu_engine* e, double bandwidth, int adaptive, int kernel, int store_s, double* betas,
                     double* betas_se, double* shat, double* qdiag, double* s)
{
    ENG_CHECK(e);
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    return guarded([&] {
        gwgpu::FitOutput o;
        e->eng.fit(bandwidth, adaptive != 0, kernel, store_s != 0, o);
        if (betas) std::memcpy(betas, o.betas.data(), sizeof(double) * o.betas.size());
        if (betas_se) std::memcpy(betas_se, o.betasSE.data(), sizeof(double) * o.betasSE.size());
        if (shat) {
            shat[0] = o.shat[0];
            shat[1] = o.shat[1];
        }
        if (qdiag) std::memcpy(qdiag, o.qdiag.data(), sizeof(double) * o.qdiag.size());
        if (s) std::memcpy(s, o.S.data(), sizeof(double) * o.S.size());
    });
}

int gwgpu_engine_max_distance(gwgpu_engine* e, double* out)
{
    ENG_CHECK(e);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    return guarded([&] { *out = e->eng.maxDistance(); });
}

int gwgpu_engine_golden(gwgpu_engine* e, int adaptive, int kernel, int criterion, double lower, double upper,
                        double* bandwidth, int* count, double* list_bw, double* list_value, int cap)
{
    ENG_CHECK(e);
    if (!bandwidth) return fail(GWGPU_ERR_INVALID, "null output");
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    return guarded([&] {
        std::map<double, double> rec;
        *bandwidth = e->eng.golden(adaptive != 0, kernel, criterion, lower, upper, rec);
        int k = 0;
        for (auto& kv : rec) {
            if (k < cap) {
                if (list_bw) list_bw[k] = kv.first;
                if (list_value) list_value[k] = kv.second;
            }
            k++;
        }
        if (count) *count = k;
    });
}

int gwgpu_engine_predict(gwgpu_engine* e, int nr, const double* locations, double bandwidth, int adaptive,
                         int kernel, double* betas)
{
    ENG_CHECK(e);
    if (nr < 1 || !locations || !betas) return fail(GWGPU_ERR_INVALID, "null argument");
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    return guarded([&] {
        std::vector<double> b;
        e->eng.predict(nr, locations, bandwidth, adaptive != 0, kernel, b);
        std::memcpy(betas, b.data(), sizeof(double) * b.size());
    });
}

int gwgpu_engine_clear_cache(gwgpu_engine* e)
{
    ENG_CHECK(e);
    return guarded([&] { e->eng.clearCaches(); });
}

int gwgpu_engine_set_distance_cache(gwgpu_engine* e, long long limit_bytes)
{
    ENG_CHECK(e);
    return guarded([&] { e->eng.setDistanceCacheLimit(limit_bytes); });
}

int gwgpu_engine_release_distance_cache(gwgpu_engine* e)
{
    ENG_CHECK(e);
    return guarded([&] { e->eng.releaseDistanceCache(); });
}

int gwgpu_engine_distance_cache_active(gwgpu_engine* e, int* active)
{
    ENG_CHECK(e);
    if (!active) return fail(GWGPU_ERR_INVALID, "null output");
    return guarded([&] { *active = e->eng.distanceCacheActive() ? 1 : 0; });
}

int gwgpu_engine_event_record(gwgpu_engine* e, int slot)
{
    ENG_CHECK(e);
    return guarded([&] { e->eng.recordEvent(slot); });
}

int gwgpu_engine_event_elapsed(gwgpu_engine* e, int first, int second, float* ms)
{
    ENG_CHECK(e);
    if (!ms) return fail(GWGPU_ERR_INVALID, "null output");
    return guarded([&] { *ms = e->eng.elapsedMs(first, second); });
}

int gwgpu_engine_thresholds(gwgpu_engine* e, double bandwidth, int adaptive, double* out)
{
    ENG_CHECK(e);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    return guarded([&] {
        std::vector<double> t;
        e->eng.thresholds(bandwidth, adaptive != 0, t);
        std::memcpy(out, t.data(), sizeof(double) * t.size());
    });
}

int gwgpu_engine_enable_stats(gwgpu_engine* e, int on)
{
    ENG_CHECK(e);
    e->eng.enableStats(on != 0, on == 2);
    return GWGPU_OK;
}

int gwgpu_engine_get_stats(gwgpu_engine* e, gwgpu_stats* out)
{
    ENG_CHECK(e);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    const gwgpu::EngineStats& s = e->eng.stats();
    out->criterion_evals = s.criterion_evals;
    out->contract_launches = s.contract_launches;
    out->contract_ms = s.contract_ms;
    out->contract_flops = s.contract_flops;
    out->contract_bytes = s.contract_bytes;
    out->select_launches = s.select_launches;
    out->select_ms = s.select_ms;
    out->kernel_launches = s.kernel_launches;
    out->contract_tiles = s.contract_tiles;
    for (int q = 0; q < 12; q++) out->contract_phase_cycles[q] = s.contract_phase_cycles[q];
    out->d2c_fills = s.d2c_fills;
    out->d2c_fill_ms = s.d2c_fill_ms;
    return GWGPU_OK;
}

int gwgpu_engine_reset_stats(gwgpu_engine* e)
{
    ENG_CHECK(e);
    e->eng.resetStats();
    return GWGPU_OK;
}

int gwgpu_engine_tc_selftest(gwgpu_engine* e, int N, const float* A, const float* B, float* D)
{
    ENG_CHECK(e);
    if (!A || !B || !D) return fail(GWGPU_ERR_INVALID, "null pointer");
    if (N < 16 || N > 256 || N % 16) return fail(GWGPU_ERR_INVALID, "N must be a multiple of 16 in [16, 256]");
    return guarded([&] { e->eng.tcSelftest(N, A, B, D); });
}

// ------------------------------------------------------------------ mgwr

#define MGWR_CHECK(g) \
    if (!(g)) return fail(GWGPU_ERR_INVALID, "null handle")

int gwgpu_mgwr_create(gwgpu_mgwr** out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null pointer");
    return guarded([&] { *out = new gwgpu_mgwr(); });
}

void gwgpu_mgwr_destroy(gwgpu_mgwr* g) { delete g; }

int gwgpu_mgwr_set_coords(gwgpu_mgwr* g, int n, const double* coords)
{
    MGWR_CHECK(g);
    if (n < 0 || (!coords && n)) return fail(GWGPU_ERR_INVALID, "bad coords");
    return guarded([&] { g->alg.setCoords(gwm::mat(n, 2, coords)); });
}

int gwgpu_mgwr_set_dependent_variable(gwgpu_mgwr* g, int n, const double* y)
{
    MGWR_CHECK(g);
    if (n < 0 || (!y && n)) return fail(GWGPU_ERR_INVALID, "bad y");
    return guarded([&] { g->alg.setDependentVariable(gwm::vec(n, 1, y)); });
}

int gwgpu_mgwr_set_independent_variables(gwgpu_mgwr* g, int n, int p, const double* x)
{
    MGWR_CHECK(g);
    if (n < 0 || p < 0 || (!x && n && p)) return fail(GWGPU_ERR_INVALID, "bad x");
    return guarded([&] { g->alg.setIndependentVariables(gwm::mat(n, p, x)); });
}

int gwgpu_mgwr_set_spatial_weights(gwgpu_mgwr* g, int p, const double* bandwidths, const int* adaptive,
                                   const int* kernels, int geographic)
{
    MGWR_CHECK(g);
    if (p < 0 || (p && (!bandwidths || !adaptive || !kernels))) return fail(GWGPU_ERR_INVALID, "bad arrays");
    for (int k = 0; k < p; k++)
        if (kernels[k] < 0 || kernels[k] > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    return guarded([&] {
        std::vector<gwm::SpatialWeight> sw;
        gwm::CRSDistance d(geographic != 0);
        for (int k = 0; k < p; k++) {
            gwm::BandwidthWeight w(bandwidths[k], adaptive[k] != 0, (gwm::BandwidthWeight::KernelFunctionType)kernels[k]);
            sw.emplace_back(&w, &d);
        }
        g->alg.setSpatialWeights(sw);
    });
}

int gwgpu_mgwr_set_bandwidth_initilize(gwgpu_mgwr* g, int p, const int* types)
{
    MGWR_CHECK(g);
    if (p < 0 || (p && !types)) return fail(GWGPU_ERR_INVALID, "bad array");
    for (int k = 0; k < p; k++)
        if (types[k] < 0 || types[k] > 2) return fail(GWGPU_ERR_INVALID, "unknown initialisation type");
    return guarded([&] {
        std::vector<gwm::GWRMultiscale::BandwidthInitilizeType> v;
        for (int k = 0; k < p; k++) v.push_back((gwm::GWRMultiscale::BandwidthInitilizeType)types[k]);
        g->alg.setBandwidthInitilize(v);
    });
}

int gwgpu_mgwr_set_bandwidth_selection_approach(gwgpu_mgwr* g, int p, const int* approaches)
{
    MGWR_CHECK(g);
    if (p < 0 || (p && !approaches)) return fail(GWGPU_ERR_INVALID, "bad array");
    for (int k = 0; k < p; k++)
        if (approaches[k] != GWGPU_MGWR_CV && approaches[k] != GWGPU_MGWR_AIC)
            return fail(GWGPU_ERR_INVALID, "unknown selection approach");
    return guarded([&] {
        std::vector<gwm::GWRMultiscale::BandwidthSelectionCriterionType> v;
        for (int k = 0; k < p; k++) v.push_back((gwm::GWRMultiscale::BandwidthSelectionCriterionType)approaches[k]);
        g->alg.setBandwidthSelectionApproach(v);
    });
}

int gwgpu_mgwr_set_preditor_centered(gwgpu_mgwr* g, int p, const int* centered)
{
    MGWR_CHECK(g);
    if (p < 0 || (p && !centered)) return fail(GWGPU_ERR_INVALID, "bad array");
    std::vector<bool> v;
    for (int k = 0; k < p; k++) v.push_back(centered[k] != 0);
    g->alg.setPreditorCentered(v);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_bandwidth_select_threshold(gwgpu_mgwr* g, int p, const double* thresholds)
{
    MGWR_CHECK(g);
    if (p < 0 || (p && !thresholds)) return fail(GWGPU_ERR_INVALID, "bad array");
    g->alg.setBandwidthSelectThreshold(std::vector<double>(thresholds, thresholds + p));
    return GWGPU_OK;
}

int gwgpu_mgwr_set_bandwidth_select_retry_times(gwgpu_mgwr* g, int times)
{
    MGWR_CHECK(g);
    if (times < 0) return fail(GWGPU_ERR_INVALID, "negative retry times");
    g->alg.setBandwidthSelectRetryTimes((std::size_t)times);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_max_iteration(gwgpu_mgwr* g, int iterations)
{
    MGWR_CHECK(g);
    if (iterations < 0) return fail(GWGPU_ERR_INVALID, "negative iteration count");
    g->alg.setMaxIteration((std::size_t)iterations);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_criterion_type(gwgpu_mgwr* g, int type)
{
    MGWR_CHECK(g);
    if (type != GWGPU_MGWR_CVR && type != GWGPU_MGWR_DCVR) return fail(GWGPU_ERR_INVALID, "unknown criterion type");
    g->alg.setCriterionType((gwm::GWRMultiscale::BackFittingCriterionType)type);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_criterion_threshold(gwgpu_mgwr* g, double threshold)
{
    MGWR_CHECK(g);
    g->alg.setCriterionThreshold(threshold);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_adaptive_lower(gwgpu_mgwr* g, int lower)
{
    MGWR_CHECK(g);
    g->alg.setAdaptiveLower(lower);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_golden_upper_bounds(gwgpu_mgwr* g, double value)
{
    MGWR_CHECK(g);
    g->alg.setGoldenUpperBounds(value);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_golden_lower_bounds(gwgpu_mgwr* g, double value)
{
    MGWR_CHECK(g);
    g->alg.setGoldenLowerBounds(value);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_has_hat_matrix(gwgpu_mgwr* g, int on)
{
    MGWR_CHECK(g);
    g->alg.setHasHatMatrix(on != 0);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_has_intercept(gwgpu_mgwr* g, int on)
{
    MGWR_CHECK(g);
    g->alg.setHasIntercept(on != 0);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_parallel_type(gwgpu_mgwr* g, int type)
{
    MGWR_CHECK(g);
    g->alg.setParallelType((gwm::ParallelType)type);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_gpu_id(gwgpu_mgwr* g, int gpu)
{
    MGWR_CHECK(g);
    g->alg.setGPUId(gpu);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_precision(gwgpu_mgwr* g, int precision)
{
    MGWR_CHECK(g);
    if (precision != GWGPU_FP64 && precision != GWGPU_MIXED) return fail(GWGPU_ERR_INVALID, "unknown precision");
    g->alg.setPrecision(precision == GWGPU_MIXED ? gwm::Precision::Mixed : gwm::Precision::FP64);
    return GWGPU_OK;
}

int gwgpu_mgwr_set_telegram(gwgpu_mgwr* g, const gwgpu_telegram* t)
{
    MGWR_CHECK(g);
    return guarded([&] {
        if (t)
            g->alg.setTelegram(std::unique_ptr<gwm::ITelegram>(new CTelegram(*t)));
        else
            g->alg.setTelegram(std::unique_ptr<gwm::ITelegram>(new gwm::Logger()));
    });
}

int gwgpu_mgwr_fit(gwgpu_mgwr* g)
{
    MGWR_CHECK(g);
    return guarded([&] { g->alg.fit(); });
}

int gwgpu_mgwr_status(gwgpu_mgwr* g)
{
    if (!g) return -1;
    return g->alg.status() == gwm::Status::Success ? GWGPU_STATUS_SUCCESS : GWGPU_STATUS_TERMINATED;
}

static int mgwr_copy(const gwm::mat& m, std::size_t n, std::size_t p, double* out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    if (m.n_elem() == 0) {
        std::fill(out, out + n * p, 0.0);
        return GWGPU_OK;
    }
    std::copy(m.memptr(), m.memptr() + m.n_elem(), out);
    return GWGPU_OK;
}

int gwgpu_mgwr_betas(gwgpu_mgwr* g, double* out)
{
    MGWR_CHECK(g);
    return mgwr_copy(g->alg.betas(), g->alg.independentVariables().n_rows, g->alg.independentVariables().n_cols, out);
}

int gwgpu_mgwr_betas_se(gwgpu_mgwr* g, double* out)
{
    MGWR_CHECK(g);
    return mgwr_copy(g->alg.betasSE(), g->alg.independentVariables().n_rows, g->alg.independentVariables().n_cols,
                     out);
}

int gwgpu_mgwr_betas_tv(gwgpu_mgwr* g, double* out)
{
    MGWR_CHECK(g);
    return mgwr_copy(g->alg.betasTV(), g->alg.independentVariables().n_rows, g->alg.independentVariables().n_cols,
                     out);
}

int gwgpu_mgwr_bandwidths(gwgpu_mgwr* g, double* out)
{
    MGWR_CHECK(g);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    const auto& sw = g->alg.spatialWeights();
    for (std::size_t k = 0; k < sw.size(); k++) out[k] = sw[k].weight()->bandwidth();
    return GWGPU_OK;
}

int gwgpu_mgwr_diagnostic(gwgpu_mgwr* g, double* out)
{
    MGWR_CHECK(g);
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    gwm::RegressionDiagnostic d = g->alg.diagnostic();
    out[0] = d.RSS;
    out[1] = d.AIC;
    out[2] = d.AICc;
    out[3] = d.ENP;
    out[4] = d.EDF;
    out[5] = d.RSquare;
    out[6] = d.RSquareAdjust;
    return GWGPU_OK;
}

int gwgpu_mgwr_info(gwgpu_mgwr* g, double* initial_bandwidth, int* iterations)
{
    MGWR_CHECK(g);
    if (initial_bandwidth) *initial_bandwidth = g->alg.initialBandwidth();
    if (iterations) *iterations = (int)g->alg.iterations();
    return GWGPU_OK;
}

int gwgpu_mgwr_counters(gwgpu_mgwr* g, long long* criterion_evals, long long* fits, long long* hat_updates,
                        long long* kernel_launches, double* seconds)
{
    MGWR_CHECK(g);
    const auto& c = g->alg.counters();
    if (criterion_evals) *criterion_evals = (long long)c.criterionEvals;
    if (fits) *fits = (long long)c.fits;
    if (hat_updates) *hat_updates = (long long)c.hatUpdates;
    if (kernel_launches) *kernel_launches = c.kernelLaunches;
    if (seconds) {
        seconds[0] = c.searchSeconds;
        seconds[1] = c.fitSeconds;
        seconds[2] = c.hatSeconds;
    }
    return GWGPU_OK;
}

}  // extern "C"
