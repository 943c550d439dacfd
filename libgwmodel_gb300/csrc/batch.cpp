// batch.cpp -- many independent GWR problems and many bandwidth candidates per
// problem in one launch per phase, replayed from a captured CUDA graph.
//
// A segment is one (problem, candidate bandwidth) pair.  Each phase covers
// every segment in a single launch: whole-row histograms (once per problem),
// the adaptive thresholds of every segment, the FP32 copy of the thresholds,
// the tcgen05 contraction (CTA = (segment, 128-row block) from a work table),
// the warp-per-location solves (block = (segment, row chunk)) and the
// fixed-order reduction per segment.  Launch count is independent of the
// number of problems and candidates, the GPU is filled even when each problem
// alone would occupy a handful of SMs, and the whole sequence is captured once
// and replayed.  An autotuner times the schedule choices on the actual batch
// (FP32 chunk length of the contraction, the order of the contraction work
// table, rows per solve block, CTAs per SM of the select) and keeps the
// fastest.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "../../include/gwgpu.h"
#include "engine.h"
#include "gw_kernels.h"

namespace gwgpu {
void set_last_error(const char* msg);

class BatchEngine {
public:
    explicit BatchEngine(int device) : device_(device)
    {
        check(cudaSetDevice(device_), "cudaSetDevice");
        check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_);
        check(cudaMallocHost(&host_sums_, sizeof(double) * (4 * kMaxSegs + 8)), "cudaMallocHost");
    }

    ~BatchEngine()
    {
        dropGraph();
        if (stream_) cudaStreamSynchronize(stream_);
        if (host_sums_) cudaFreeHost(host_sums_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    static constexpr int kMaxSegs = 1 << 16;

    struct Tuning {
        int flush_tiles = 64;  // FP32 chunk of the contraction
        int order = 1;         // 0: segment-major work table, 1: heaviest row blocks first
        int solve_rows = 32;   // rows per solve block
        int select_ctas = 12;  // select CTAs per SM
    };

    void setProblems(int count, const int* n, const int* p, const double* const* x, const double* const* y,
                     const double* const* coords, const int* geographic, int precision)
    {
        if (count < 1) throw std::invalid_argument("need at least one problem");
        check(cudaSetDevice(device_), "cudaSetDevice");
        dropGraph();
        precision_ = precision;
        eng_.clear();
        for (int q = 0; q < count; q++) {
            std::unique_ptr<Engine> e(new Engine(device_));
            e->setData(n[q], p[q], x[q], y[q], coords[q], geographic[q] != 0);
            e->setPrecision(precision);
            if (precision == kMixed) e->ensureMixed();
            eng_.push_back(std::move(e));
        }
        hist_ready_ = false;
        segs_.clear();
    }

    void setCandidates(const int* counts, const double* const* bws, bool adaptive, int kernel, int criterion)
    {
        if (eng_.empty()) throw std::logic_error("no problems");
        if (kernel < 0 || kernel > 4) throw std::invalid_argument("unknown kernel");
        if (criterion != kAIC && criterion != kCV) throw std::invalid_argument("unknown criterion");
        dropGraph();
        segs_.clear();
        for (size_t q = 0; q < eng_.size(); q++) {
            for (int c = 0; c < counts[q]; c++) {
                const double bw = bws[q][c];
                if (adaptive) {
                    if (bw != std::floor(bw) || bw < 1 || bw > eng_[q]->n())
                        throw std::invalid_argument("adaptive candidates must be whole neighbour counts in [1, n]");
                } else if (!(bw > 0)) {
                    throw std::invalid_argument("fixed candidates must be positive");
                }
                segs_.push_back(Seg{(int)q, bw});
            }
        }
        if ((int)segs_.size() > kMaxSegs) throw std::invalid_argument("too many (problem, candidate) pairs");
        adaptive_ = adaptive;
        kernel_ = kernel;
        criterion_ = criterion;
        build();
    }

    // Criterion value of every segment (DBL_MAX where a local system failed).
    void evaluate(double* values, bool use_graph)
    {
        if (segs_.empty()) throw std::logic_error("no candidates");
        check(cudaSetDevice(device_), "cudaSetDevice");
        ensureHist();
        auto t0 = std::chrono::steady_clock::now();
        if (use_graph) {
            if (!exec_) capture();
            check(cudaGraphLaunch(exec_, stream_), "cudaGraphLaunch");
        } else {
            enqueue();
        }
        check(cudaStreamSynchronize(stream_), "evaluate");
        last_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        int err[2] = {0, 0};
        std::memcpy(err, host_sums_ + 4 * segs_.size(), sizeof(err));
        if (err[0]) throw CudaError("batched threshold select failed (code " + std::to_string(err[0]) + ")");
        if (err[1]) throw CudaError("batched tensor-core contraction: a bounded wait timed out");
        for (size_t s = 0; s < segs_.size(); s++) {
            const double* v = host_sums_ + 4 * s;
            const Engine& e = *eng_[segs_[s].q];
            double rss = v[1];
            if (precision_ == kMixed) rss *= e.s_y_ * e.s_y_;
            double out;
            if (v[3] > 0.0) out = DBL_MAX;
            else if (criterion_ == kCV) out = rss;
            else {
                const double n = (double)e.n_, trS = v[0];
                out = n * std::log(rss / n) + n * std::log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
            }
            values[s] = std::isfinite(out) ? out : DBL_MAX;
        }
        evaluations_++;
    }

    // Times every schedule variant (median of `repeats` uncaptured runs each)
    // and keeps the fastest; the graph is recaptured for it.
    void autotune(int repeats)
    {
        if (segs_.empty()) throw std::logic_error("no candidates");
        std::vector<double> vals(segs_.size());
        ensureHist();
        std::vector<Tuning> cands;
        const int flushes[] = {32, 64};
        const int orders[] = {0, 1};
        const int rows[] = {16, 32, 64};
        const int ctas[] = {8, 12, 16};
        for (int f : flushes)
            for (int o : orders)
                cands.push_back(Tuning{f, o, tune_.solve_rows, tune_.select_ctas});
        double best = 1e300;
        Tuning bestT = tune_;
        auto timeit = [&](const Tuning& t) {
            tune_ = t;
            dropGraph();
            build();
            std::vector<double> ms;
            for (int r = 0; r < std::max(1, repeats); r++) {
                evaluate(vals.data(), false);
                ms.push_back(last_ms_);
            }
            std::sort(ms.begin(), ms.end());
            return ms[ms.size() / 2];
        };
        // contraction schedule first, then solve chunking and select width on the winner
        for (const Tuning& t : cands) {
            const double m = timeit(t);
            if (m < best) best = m, bestT = t;
        }
        for (int r : rows) {
            Tuning t = bestT;
            t.solve_rows = r;
            const double m = timeit(t);
            if (m < best) best = m, bestT = t;
        }
        for (int c : ctas) {
            Tuning t = bestT;
            t.select_ctas = c;
            const double m = timeit(t);
            if (m < best) best = m, bestT = t;
        }
        tune_ = bestT;
        tuned_ms_ = best;
        tuned_ = true;
        dropGraph();
        build();
    }

    void setTuning(const Tuning& t)
    {
        if (t.flush_tiles < 2 || t.solve_rows < 4 || t.select_ctas < 1) throw std::invalid_argument("bad tuning");
        tune_ = t;
        dropGraph();
        if (!segs_.empty()) build();
    }

    void info(gwgpu_batch_info* o) const
    {
        std::memset(o, 0, sizeof(*o));
        o->problems = (int)eng_.size();
        o->segments = (int)segs_.size();
        o->flush_tiles = tune_.flush_tiles;
        o->order = tune_.order;
        o->solve_rows = tune_.solve_rows;
        o->select_ctas = tune_.select_ctas;
        o->tuned = tuned_ ? 1 : 0;
        o->tuned_ms = tuned_ms_;
        o->last_ms = last_ms_;
        o->graph = exec_ ? 1 : 0;
        o->launches_per_evaluate = launches_;
        o->contract_ctas = (int)tc_work_.size();
        o->rows_total = (double)rows_total_;
    }

private:
    struct Seg {
        int q;
        double bw;
    };

    void dropGraph()
    {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
        exec_ = nullptr;
        graph_ = nullptr;
    }

    // Whole-row histogram caches of every problem (once per dataset).
    void ensureHist()
    {
        if (hist_ready_ || !adaptive_) return;
        for (int geo = 0; geo < 2; geo++) {
            std::vector<SelectArgs> args;
            std::vector<long long> start{0};
            for (auto& e : eng_) {
                if (e->geographic_ != (geo == 1)) continue;
                e->hist_.alloc((size_t)e->n_ * 4096);
                e->hcoarse_.alloc((size_t)e->n_ * 64);
                e->hist_tried_ = true;
                SelectArgs a = selectArgs(*e, 1, nullptr);
                args.push_back(a);
                start.push_back(start.back() + (e->n_ + kSelHistRows - 1) / kSelHistRows);
            }
            if (args.empty()) continue;
            DevBuf<SelectArgs> da;
            DevBuf<long long> ds;
            upload(da, args);
            upload(ds, start);
            check(launch_select_hist_batch(da.get(), ds.get(), (int)args.size(), geo == 1, num_sms_, stream_),
                  "batched histograms");
            check(cudaStreamSynchronize(stream_), "histograms");
        }
        for (auto& e : eng_) e->hist_valid_ = true;
        hist_ready_ = true;
        // the select argument tables were built before the caches existed (null
        // cache pointers make every select scan whole rows): rebuild them
        dropGraph();
        build();
    }

    SelectArgs selectArgs(Engine& e, unsigned rank, double* out)
    {
        SelectArgs a{};
        a.n = e.n_;
        a.ntiles = e.ntiles32_;
        a.P = e.points();
        a.pts = e.pts32_.get();
        a.tb = e.tbsel_.get();
        a.stb = e.stb_.get();
        a.hist_cache = e.hist_.get();
        a.cache_valid = 1;
        a.hist_coarse = e.hcoarse_.get();
        a.rank = rank;
        a.dlo = e.dlo_;
        a.dhi = e.dhi_;
        a.eps = e.sel_eps_;
        a.delta = e.sel_delta_;
        a.out = out;
        a.err = err_.get();
        return a;
    }

    template <class T>
    void upload(DevBuf<T>& d, const std::vector<T>& h)
    {
        d.alloc(h.size());
        check(cudaMemcpyAsync(d.get(), h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, stream_), "H2D");
    }

    // Per-segment buffers, argument tables and work tables.
    void build()
    {
        const size_t S = segs_.size();
        err_.alloc(2);
        // offsets of every per-row array
        std::vector<size_t> off_row(S + 1, 0), off_g(S + 1, 0), off_acc(S + 1, 0);
        for (size_t s = 0; s < S; s++) {
            const Engine& e = *eng_[segs_[s].q];
            off_row[s + 1] = off_row[s] + e.n_;
            off_g[s + 1] = off_g[s] + (size_t)e.n_ * e.m_;
            // rows in groups of 128 (the contraction's layout)
            off_acc[s + 1] = off_acc[s] + (precision_ == kMixed ? (size_t)(e.n_ + 127) / 128 * 128 * e.npad_ : 0);
        }
        rows_total_ = off_row[S];
        seg_g_.resize(S);
        thr_.alloc(off_row[S]);
        thr32_.alloc(precision_ == kMixed ? off_row[S] : 1);
        G_.alloc(off_g[S]);
        for (size_t s = 0; s < S; s++) seg_g_[s] = G_.get() + off_g[s];
        acc_.alloc(std::max<size_t>(off_acc[S], 1));
        sii_.alloc(off_row[S]);
        resid_.alloc(off_row[S]);
        const int R = tune_.solve_rows;
        std::vector<int> first(S + 1, 0);
        for (size_t s = 0; s < S; s++) first[s + 1] = first[s] + (eng_[segs_[s].q]->n_ + R - 1) / R;
        part_.alloc((size_t)first[S] * 4 + 4);
        sums_.alloc(4 * S + 2);
        launches_ = 0;

        // selects and their FP32 copies (adaptive only)
        sel_args_.assign(2, {});
        sel_start_.assign(2, {0});
        tf_in_.clear();
        tf_out_.clear();
        tf_start_.assign(1, 0);
        if (adaptive_) {
            for (size_t s = 0; s < S; s++) {
                Engine& e = *eng_[segs_[s].q];
                const int geo = e.geographic_ ? 1 : 0;
                sel_args_[geo].push_back(selectArgs(e, (unsigned)segs_[s].bw, thr_.get() + off_row[s]));
                sel_start_[geo].push_back(sel_start_[geo].back() + e.n_);
                if (precision_ == kMixed) {
                    tf_in_.push_back(thr_.get() + off_row[s]);
                    tf_out_.push_back(thr32_.get() + off_row[s]);
                    tf_start_.push_back(tf_start_.back() + e.n_);
                }
            }
            for (int geo = 0; geo < 2; geo++) {
                if (sel_args_[geo].empty()) continue;
                upload(d_sel_[geo], sel_args_[geo]);
                upload(d_sel_start_[geo], sel_start_[geo]);
                launches_++;
            }
            if (!tf_in_.empty()) {
                upload(d_tf_in_, tf_in_);
                upload(d_tf_out_, tf_out_);
                upload(d_tf_start_, tf_start_);
                launches_++;
            }
        }

        // contractions
        tc_args_.clear();
        tc_work_.clear();
        tc_work_geo_.assign(2, {});
        max_npad_ = 64;
        max_ntiles_ = 1;
        if (precision_ == kMixed) {
            std::vector<std::pair<double, int2>> items[2];
            for (size_t s = 0; s < S; s++) {
                Engine& e = *eng_[segs_[s].q];
                TcArgs a{};
                a.n = e.n_;
                a.mcols = e.m_;
                a.npad = e.npad_;
                a.ntiles = e.ntiles32_;
                a.pts = e.pts32_.get();
                a.tb = e.tbsel_.get();
                a.zimg = e.zimg_.get();
                a.thr = adaptive_ ? thr32_.get() + off_row[s] : nullptr;
                a.bw = (float)segs_[s].bw;
                a.kernel = kernel_;
                a.exclude_self = criterion_ == kCV ? 1 : 0;
                a.skip = 1;
                a.flush_tiles = tune_.flush_tiles;
                a.wpow = 1;
                a.acc = acc_.get() + off_acc[s];
                a.G = G_.get() + off_g[s];
                a.ldg = e.m_;
                a.err = err_.get() + 1;
                tc_args_.push_back(a);
                max_npad_ = std::max(max_npad_, e.npad_);
                max_ntiles_ = std::max(max_ntiles_, e.ntiles32_);
                // work estimate of a row block: neighbours x columns (the dense bound for fixed kernels)
                const double nb = adaptive_ ? std::min(segs_[s].bw, (double)e.n_) : (double)e.n_;
                const double w = nb * e.npad_;
                for (int r0 = 0; r0 < e.n_; r0 += 128)
                    items[e.geographic_ ? 1 : 0].push_back({w, make_int2((int)s, r0)});
            }
            for (int geo = 0; geo < 2; geo++) {
                if (tune_.order == 1)
                    std::stable_sort(items[geo].begin(), items[geo].end(),
                                     [](const auto& a, const auto& b) { return a.first > b.first; });
                for (auto& it : items[geo]) tc_work_geo_[geo].push_back(it.second);
            }
            upload(d_tc_, tc_args_);
            for (int geo = 0; geo < 2; geo++) {
                if (tc_work_geo_[geo].empty()) continue;
                upload(d_tc_work_[geo], tc_work_geo_[geo]);
                launches_++;
                tc_work_.insert(tc_work_.end(), tc_work_geo_[geo].begin(), tc_work_geo_[geo].end());
            }
        } else {
            launches_ += (int)S;  // one FP64 contraction per segment
        }

        // solves and reductions
        sv_args_.clear();
        sv_work_.clear();
        max_p_ = 1;
        for (size_t s = 0; s < S; s++) {
            Engine& e = *eng_[segs_[s].q];
            const bool mixed = precision_ == kMixed;
            SolveArgs a{};
            a.n = e.n_;
            a.p = e.p_;
            a.mode = criterion_ == kCV ? kSolveCV : kSolveAIC;
            a.kernel = kernel_;
            a.G = G_.get() + off_g[s];
            a.ldg = e.m_;
            a.X = mixed ? e.xs_.get() : e.x_.get();
            a.y = mixed ? e.ys_.get() : e.y_.get();
            a.thr = adaptive_ ? thr_.get() + off_row[s] : nullptr;
            a.bw = segs_[s].bw;
            a.beta = nullptr;  // criteria only: no coefficients
            a.sii = sii_.get() + off_row[s];
            a.resid = resid_.get() + off_row[s];
            a.partials = part_.get() + (size_t)first[s] * 4;
            a.tcol = -1;
            sv_args_.push_back(a);
            max_p_ = std::max(max_p_, e.p_);
            int slot = 0;
            for (int r0 = 0; r0 < e.n_; r0 += R, slot++) sv_work_.push_back(make_int4((int)s, r0, std::min(e.n_, r0 + R), slot));
        }
        upload(d_sv_, sv_args_);
        upload(d_sv_work_, sv_work_);
        upload(d_first_, first);
        launches_ += 2;
        check(cudaStreamSynchronize(stream_), "batch build");
    }

    // Every phase of one evaluation on the stream (no host synchronisation).
    void enqueue()
    {
        const size_t S = segs_.size();
        check(cudaMemsetAsync(err_.get(), 0, 2 * sizeof(int), stream_), "memset err");
        if (adaptive_) {
            for (int geo = 0; geo < 2; geo++) {
                if (sel_args_[geo].empty()) continue;
                check(launch_select_batch(d_sel_[geo].get(), d_sel_start_[geo].get(), (int)sel_args_[geo].size(),
                                          geo == 1, precision_ == kFP64, num_sms_ * tune_.select_ctas / 12, stream_),
                      "batched select");
            }
            if (!tf_in_.empty())
                check(launch_to_float_batch(d_tf_in_.get(), d_tf_out_.get(), d_tf_start_.get(), (int)tf_in_.size(),
                                            num_sms_, stream_),
                      "batched thr32");
        }
        if (precision_ == kMixed) {
            for (int geo = 0; geo < 2; geo++) {
                if (tc_work_geo_[geo].empty()) continue;
                check(launch_contract_tc_batch(d_tc_.get(), d_tc_work_[geo].get(), (int)tc_work_geo_[geo].size(),
                                               max_npad_, max_ntiles_, tune_.flush_tiles, geo == 1, kernel_, stream_),
                      "batched contraction");
            }
        } else {
            for (size_t s = 0; s < S; s++) {
                Engine& e = *eng_[segs_[s].q];
                check(launch_contract64(e.points(), e.geographic_, e.tb16_.get(), e.z_.get(), e.m_, e.m_, seg_g_[s],
                                        e.m_, sv_args_[s].thr, segs_[s].bw, kernel_, criterion_ == kCV, 1, true,
                                        stream_),
                      "contract64");
            }
        }
        check(launch_solve_batch(d_sv_.get(), d_sv_work_.get(), (int)sv_work_.size(),
                                 criterion_ == kCV ? kSolveCV : kSolveAIC, max_p_, stream_),
              "batched solve");
        check(launch_reduce_batch(part_.get(), d_first_.get(), (int)S, sums_.get(), stream_), "batched reduce");
        check(cudaMemcpyAsync(sums_.get() + 4 * S, err_.get(), 2 * sizeof(int), cudaMemcpyDeviceToDevice, stream_),
              "err");
        check(cudaMemcpyAsync(host_sums_, sums_.get(), sizeof(double) * (4 * S + 1), cudaMemcpyDeviceToHost, stream_),
              "D2H sums");
    }

    void capture()
    {
        dropGraph();
        // one uncaptured pass first, so every kernel attribute is set before capture
        enqueue();
        check(cudaStreamSynchronize(stream_), "pre-capture");
        check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed), "begin capture");
        enqueue();
        check(cudaStreamEndCapture(stream_, &graph_), "end capture");
        check(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate");
    }

    int device_;
    cudaStream_t stream_ = nullptr;
    int num_sms_ = 0;
    int precision_ = kMixed;
    std::vector<std::unique_ptr<Engine>> eng_;
    std::vector<Seg> segs_;
    bool adaptive_ = true, hist_ready_ = false, tuned_ = false;
    int kernel_ = GW_KERNEL_BISQUARE, criterion_ = kAIC;
    Tuning tune_;
    double last_ms_ = 0.0, tuned_ms_ = 0.0;
    long long evaluations_ = 0;
    int launches_ = 0, max_npad_ = 64, max_ntiles_ = 1, max_p_ = 1;
    size_t rows_total_ = 0;
    double* host_sums_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;

    DevBuf<double> thr_, G_, sii_, resid_, part_, sums_;
    DevBuf<float> thr32_;
    DevBuf<float2> acc_;
    DevBuf<int> err_, d_first_;
    std::vector<std::vector<SelectArgs>> sel_args_;
    std::vector<std::vector<long long>> sel_start_;
    DevBuf<SelectArgs> d_sel_[2];
    DevBuf<long long> d_sel_start_[2];
    std::vector<const double*> tf_in_;
    std::vector<float*> tf_out_;
    std::vector<long long> tf_start_;
    DevBuf<const double*> d_tf_in_;
    DevBuf<float*> d_tf_out_;
    DevBuf<long long> d_tf_start_;
    std::vector<TcArgs> tc_args_;
    std::vector<int2> tc_work_;
    std::vector<std::vector<int2>> tc_work_geo_;
    DevBuf<TcArgs> d_tc_;
    DevBuf<int2> d_tc_work_[2];
    std::vector<SolveArgs> sv_args_;
    std::vector<double*> seg_g_;
    std::vector<int4> sv_work_;
    DevBuf<SolveArgs> d_sv_;
    DevBuf<int4> d_sv_work_;
};

}  // namespace gwgpu

struct gwgpu_batch {
    std::unique_ptr<gwgpu::BatchEngine> impl;
};

namespace {

int fail(int code, const char* msg)
{
    gwgpu::set_last_error(msg);
    return code;
}

template <class F>
int guarded(F&& f)
{
    try {
        f();
    } catch (const gwgpu::NotSPDError& ex) {
        return fail(GWGPU_ERR_NOT_SPD, ex.what());
    } catch (const gwgpu::CudaError& ex) {
        return fail(GWGPU_ERR_CUDA, ex.what());
    } catch (const std::invalid_argument& ex) {
        return fail(GWGPU_ERR_INVALID, ex.what());
    } catch (const std::logic_error& ex) {
        return fail(GWGPU_ERR_INVALID, ex.what());
    } catch (const std::exception& ex) {
        return fail(GWGPU_ERR_RUNTIME, ex.what());
    }
    return GWGPU_OK;
}

}  // namespace

extern "C" {

int gwgpu_batch_create(int device, gwgpu_batch** out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    int count = 0;
    cudaError_t rc = cudaGetDeviceCount(&count);
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    if (device < 0 || device >= count) return fail(GWGPU_ERR_INVALID, "no such device");
    return guarded([&] { *out = new gwgpu_batch{std::unique_ptr<gwgpu::BatchEngine>(new gwgpu::BatchEngine(device))}; });
}

int gwgpu_batch_destroy(gwgpu_batch* b)
{
    if (!b) return fail(GWGPU_ERR_INVALID, "null batch");
    delete b;
    return GWGPU_OK;
}

int gwgpu_batch_set_problems(gwgpu_batch* b, int count, const int* n, const int* p, const double* const* x,
                             const double* const* y, const double* const* coords, const int* geographic,
                             int precision)
{
    if (!b || !n || !p || !x || !y || !coords || !geographic) return fail(GWGPU_ERR_INVALID, "null argument");
    if (precision != GWGPU_FP64 && precision != GWGPU_MIXED) return fail(GWGPU_ERR_INVALID, "unknown precision");
    for (int q = 0; q < count; q++)
        if (n[q] < 3 || p[q] < 1 || p[q] > gwgpu::kMaxP || !x[q] || !y[q] || !coords[q])
            return fail(GWGPU_ERR_INVALID, "each problem needs n >= 3, p in [1, 32] and data");
    return guarded([&] { b->impl->setProblems(count, n, p, x, y, coords, geographic, precision); });
}

int gwgpu_batch_set_candidates(gwgpu_batch* b, const int* counts, const double* const* bandwidths, int adaptive,
                               int kernel, int criterion)
{
    if (!b || !counts || !bandwidths) return fail(GWGPU_ERR_INVALID, "null argument");
    return guarded([&] { b->impl->setCandidates(counts, bandwidths, adaptive != 0, kernel, criterion); });
}

int gwgpu_batch_evaluate(gwgpu_batch* b, int use_graph, double* values)
{
    if (!b || !values) return fail(GWGPU_ERR_INVALID, "null argument");
    return guarded([&] { b->impl->evaluate(values, use_graph != 0); });
}

int gwgpu_batch_autotune(gwgpu_batch* b, int repeats)
{
    if (!b) return fail(GWGPU_ERR_INVALID, "null batch");
    return guarded([&] { b->impl->autotune(repeats); });
}

int gwgpu_batch_set_tuning(gwgpu_batch* b, int flush_tiles, int order, int solve_rows, int select_ctas)
{
    if (!b) return fail(GWGPU_ERR_INVALID, "null batch");
    return guarded([&] {
        b->impl->setTuning(gwgpu::BatchEngine::Tuning{flush_tiles, order, solve_rows, select_ctas});
    });
}

int gwgpu_batch_get_info(gwgpu_batch* b, gwgpu_batch_info* out)
{
    if (!b || !out) return fail(GWGPU_ERR_INVALID, "null argument");
    b->impl->info(out);
    return GWGPU_OK;
}

}  // extern "C"
