// server.cpp -- the serving loop: independent GWR fits and bandwidth searches
// on one GPU, admitted as worker slots and the HBM budget allow, each slot an
// engine on its own stream so that requests overlap on the device.
//
// A slot's engine is long-lived: its buffers grow to the largest dataset the
// slot has served and are reused, so steady-state serving allocates nothing
// (cudaMalloc and cudaFree would synchronise the whole device and stall the
// other slots).  Memory held by a slot counts against the budget until the
// slot is trimmed; an idle slot trims itself when its memory is what keeps
// the oldest waiting request out.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gwgpu.h"
#include "engine.h"
#include "gw_kernels.h"

namespace gwgpu {
void set_last_error(const char* msg);

namespace {

// First fit among idle slots: no growth if some slot already holds enough
// (the smallest such), else the idle slot holding the most (least growth).
int admit_slot(double budget, int slots, const double* reserved, const int* busy, double estimate)
{
    double total = 0.0;
    for (int s = 0; s < slots; s++) total += reserved[s];
    int best = -1;
    for (int s = 0; s < slots; s++) {
        if (busy[s]) continue;
        const double after = total - reserved[s] + std::max(reserved[s], estimate);
        if (after > budget) continue;
        if (best < 0) {
            best = s;
            continue;
        }
        const bool fits_s = reserved[s] >= estimate, fits_b = reserved[best] >= estimate;
        if (fits_s != fits_b) {
            if (fits_s) best = s;
        } else if (fits_s ? reserved[s] < reserved[best] : reserved[s] > reserved[best]) {
            best = s;
        }
    }
    return best;
}

struct Request {
    long long id = 0;
    gwgpu_request spec{};
    std::vector<double> x, y, coords;
    double* betas_out = nullptr;
    double estimate = 0.0;
    gwgpu_result res{};
    bool done = false;
};

double now_ms(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

class Server {
public:
    Server(int device, double budget, int slots)
        : device_(device), budget_(budget), slots_(slots), reserved_(slots, 0.0), busy_(slots, 0),
          engines_(slots), t0_(std::chrono::steady_clock::now())
    {
        for (int s = 0; s < slots; s++) threads_.emplace_back([this, s] { worker(s); });
    }

    ~Server()
    {
        {
            std::unique_lock<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        for (auto& t : threads_) t.join();
    }

    long long submit(const gwgpu_request& r, double* betas_out)
    {
        auto q = std::make_shared<Request>();
        q->spec = r;
        const size_t n = (size_t)r.n, p = (size_t)r.p;
        q->x.assign(r.x, r.x + n * p);
        q->y.assign(r.y, r.y + n);
        q->coords.assign(r.coords, r.coords + 2 * n);
        q->spec.x = q->spec.y = q->spec.coords = nullptr;
        q->betas_out = betas_out;
        q->estimate = estimate(r);
        std::unique_lock<std::mutex> lk(mu_);
        q->id = ++next_id_;
        q->res.submit_ms = now_ms(t0_);
        q->res.slot = -1;
        all_[q->id] = q;
        submitted_++;
        if (q->estimate > budget_) {
            q->res.status = GWGPU_ERR_REJECTED;
            std::snprintf(q->res.error, sizeof(q->res.error), "request needs ~%.3g GB, budget %.3g GB",
                          q->estimate / 1e9, budget_ / 1e9);
            q->res.end_ms = q->res.start_ms = q->res.submit_ms;
            q->done = true;
            rejected_++;
            cv_done_.notify_all();
            return q->id;
        }
        queue_.push_back(q);
        lk.unlock();
        cv_work_.notify_all();
        return q->id;
    }

    double estimate(const gwgpu_request& r) const
    {
        return (double)Engine::estimateBytes(r.n, r.p, r.geographic != 0, r.precision == GWGPU_MIXED, r.adaptive != 0,
                                             hist_limit(r.n));
    }

    // 0: done (out filled), 1: timed out, -1: unknown id
    int wait(long long id, double timeout_ms, gwgpu_result* out)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) return -1;
        auto q = it->second;
        auto ready = [&] { return q->done; };
        if (timeout_ms < 0) {
            cv_done_.wait(lk, ready);
        } else if (!cv_done_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
            return 1;
        }
        if (out) *out = q->res;
        all_.erase(id);
        return 0;
    }

    int poll(long long id, int* done)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) return -1;
        *done = it->second->done ? 1 : 0;
        return 0;
    }

    void stats(gwgpu_server_stats* o)
    {
        std::unique_lock<std::mutex> lk(mu_);
        std::memset(o, 0, sizeof(*o));
        o->submitted = submitted_;
        o->completed = (long long)lat_.size();
        o->failed = failed_;
        o->rejected = rejected_;
        o->queued = (long long)queue_.size();
        for (int s = 0; s < slots_; s++) o->running += busy_[s];
        std::vector<double> l = lat_;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) {
            if (l.empty()) return 0.0;
            const double pos = q * (double)(l.size() - 1);
            const size_t i = (size_t)pos;
            const double f = pos - (double)i;
            return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
        };
        o->p50_ms = pct(0.50);
        o->p99_ms = pct(0.99);
        double sum = 0.0;
        for (double v : l) sum += v;
        o->mean_ms = l.empty() ? 0.0 : sum / (double)l.size();
        o->first_start_ms = first_start_ < 0 ? 0.0 : first_start_;
        o->last_end_ms = last_end_;
        o->local_fits = local_fits_;
        for (double r : reserved_) o->reserved_bytes += r;
        o->peak_reserved_bytes = peak_reserved_;
        o->max_concurrent = max_concurrent_;
    }

private:
    // The histogram cache of a slot is limited to an eighth of the budget.
    long long hist_limit(int) const { return (long long)(budget_ / 8); }

    void worker(int slot)
    {
        cudaSetDevice(device_);
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            std::shared_ptr<Request> q;
            for (;;) {
                if (stop_ && queue_.empty()) return;
                if (!queue_.empty()) {
                    const double est = queue_.front()->estimate;
                    const int s = admit_slot(budget_, slots_, reserved_.data(), busy_.data(), est);
                    if (s == slot) {
                        q = queue_.front();
                        queue_.pop_front();
                        break;
                    }
                    if (s < 0 && reserved_[slot] > 0.0 && !busy_[slot]) {
                        // memory is what blocks the oldest request: give this idle slot's back
                        busy_[slot] = 1;
                        lk.unlock();
                        engines_[slot].reset();
                        lk.lock();
                        busy_[slot] = 0;
                        reserved_[slot] = 0.0;
                        cv_work_.notify_all();
                        continue;
                    }
                    if (s >= 0) {
                        // another idle slot is the better fit; make sure it looks
                        cv_work_.notify_all();
                    }
                }
                cv_work_.wait(lk);
            }
            busy_[slot] = 1;
            reserved_[slot] = std::max(reserved_[slot], q->estimate);
            double total = 0.0;
            int running = 0;
            for (int s = 0; s < slots_; s++) {
                total += reserved_[s];
                running += busy_[s];
            }
            peak_reserved_ = std::max(peak_reserved_, total);
            max_concurrent_ = std::max(max_concurrent_, running);
            q->res.slot = slot;
            q->res.start_ms = now_ms(t0_);
            if (first_start_ < 0) first_start_ = q->res.start_ms;
            lk.unlock();
            run(slot, *q);
            lk.lock();
            q->res.end_ms = now_ms(t0_);
            last_end_ = std::max(last_end_, q->res.end_ms);
            if (q->res.status == GWGPU_OK) {
                lat_.push_back(q->res.end_ms - q->res.submit_ms);
                local_fits_ += (double)q->spec.n * (q->res.evaluations + 1);
            } else {
                failed_++;
            }
            busy_[slot] = 0;
            q->done = true;
            cv_done_.notify_all();
            cv_work_.notify_all();
        }
    }

    void run(int slot, Request& q)
    {
        const gwgpu_request& r = q.spec;
        try {
            if (!engines_[slot]) engines_[slot].reset(new Engine(device_));
            Engine& e = *engines_[slot];
            e.setHistLimit(hist_limit(r.n));
            e.setDistanceCacheLimit(0);  // n^2 bytes per request would break the HBM budget's admission
            e.setData(r.n, r.p, q.x.data(), q.y.data(), q.coords.data(), r.geographic != 0);
            e.setPrecision(r.precision == GWGPU_MIXED ? kMixed : kFP64);
            double bw = r.bandwidth;
            int evals = 0;
            if (r.kind == GWGPU_REQ_SEARCH) {
                const double lower = r.adaptive ? 20.0 : 0.0;
                const double upper = r.adaptive ? (double)r.n : e.maxDistance();
                std::map<double, double> rec;
                bw = e.golden(r.adaptive != 0, r.kernel, r.criterion, lower, upper, rec);
                evals = (int)rec.size();
            }
            FitOutput out;
            e.fit(bw, r.adaptive != 0, r.kernel, false, out);
            const double n = (double)r.n, trS = out.shat[0];
            q.res.aicc = n * std::log(out.rss / n) + n * std::log(2 * M_PI) + n * ((n + trS) / (n - 2 - trS));
            q.res.rss = out.rss;
            q.res.shat[0] = out.shat[0];
            q.res.shat[1] = out.shat[1];
            q.res.bandwidth = bw;
            q.res.evaluations = evals;
            if (q.betas_out) std::memcpy(q.betas_out, out.betas.data(), sizeof(double) * out.betas.size());
            q.res.status = GWGPU_OK;
        } catch (const NotSPDError& ex) {
            q.res.status = GWGPU_ERR_NOT_SPD;
            std::snprintf(q.res.error, sizeof(q.res.error), "%s", ex.what());
        } catch (const CudaError& ex) {
            q.res.status = GWGPU_ERR_CUDA;
            std::snprintf(q.res.error, sizeof(q.res.error), "%s", ex.what());
        } catch (const std::invalid_argument& ex) {
            q.res.status = GWGPU_ERR_INVALID;
            std::snprintf(q.res.error, sizeof(q.res.error), "%s", ex.what());
        } catch (const std::exception& ex) {
            q.res.status = GWGPU_ERR_RUNTIME;
            std::snprintf(q.res.error, sizeof(q.res.error), "%s", ex.what());
        }
    }

    const int device_;
    const double budget_;
    const int slots_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<std::shared_ptr<Request>> queue_;
    std::unordered_map<long long, std::shared_ptr<Request>> all_;
    std::vector<double> reserved_;
    std::vector<int> busy_;
    std::vector<std::unique_ptr<Engine>> engines_;
    std::vector<std::thread> threads_;
    std::chrono::steady_clock::time_point t0_;
    bool stop_ = false;
    long long next_id_ = 0, submitted_ = 0, failed_ = 0, rejected_ = 0;
    std::vector<double> lat_;
    double first_start_ = -1.0, last_end_ = 0.0, local_fits_ = 0.0, peak_reserved_ = 0.0;
    int max_concurrent_ = 0;
};

}  // namespace gwgpu

struct gwgpu_server {
    std::unique_ptr<gwgpu::Server> impl;
};

namespace {

int fail(int code, const char* msg)
{
    gwgpu::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" {

int gwgpu_server_create(int device, double hbm_budget_bytes, int slots, gwgpu_server** out)
{
    if (!out) return fail(GWGPU_ERR_INVALID, "null output");
    if (slots < 1 || slots > 64) return fail(GWGPU_ERR_INVALID, "slots must be in [1, 64]");
    if (!(hbm_budget_bytes > 0)) return fail(GWGPU_ERR_INVALID, "HBM budget must be positive");
    int count = 0;
    cudaError_t rc = cudaGetDeviceCount(&count);
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    if (device < 0 || device >= count) return fail(GWGPU_ERR_INVALID, "no such device");
    try {
        *out = new gwgpu_server{std::unique_ptr<gwgpu::Server>(new gwgpu::Server(device, hbm_budget_bytes, slots))};
    } catch (const std::exception& ex) {
        return fail(GWGPU_ERR_RUNTIME, ex.what());
    }
    return GWGPU_OK;
}

int gwgpu_server_destroy(gwgpu_server* s)
{
    if (!s) return fail(GWGPU_ERR_INVALID, "null server");
    delete s;
    return GWGPU_OK;
}

int gwgpu_server_submit(gwgpu_server* s, const gwgpu_request* r, double* betas_out, long long* id)
{
    if (!s || !r || !id) return fail(GWGPU_ERR_INVALID, "null argument");
    if (r->n < 3 || r->p < 1 || r->p > gwgpu::kMaxP) return fail(GWGPU_ERR_INVALID, "need n >= 3 and p in [1, 32]");
    if (!r->x || !r->y || !r->coords) return fail(GWGPU_ERR_INVALID, "null data");
    if (r->kind != GWGPU_REQ_FIT && r->kind != GWGPU_REQ_SEARCH) return fail(GWGPU_ERR_INVALID, "unknown kind");
    if (r->kernel < 0 || r->kernel > 4) return fail(GWGPU_ERR_INVALID, "unknown kernel");
    if (r->criterion != GWGPU_AIC && r->criterion != GWGPU_CV) return fail(GWGPU_ERR_INVALID, "unknown criterion");
    if (r->precision != GWGPU_FP64 && r->precision != GWGPU_MIXED) return fail(GWGPU_ERR_INVALID, "unknown precision");
    if (r->kind == GWGPU_REQ_FIT && !(r->bandwidth > 0)) return fail(GWGPU_ERR_INVALID, "bandwidth must be positive");
    try {
        *id = s->impl->submit(*r, betas_out);
    } catch (const std::exception& ex) {
        return fail(GWGPU_ERR_RUNTIME, ex.what());
    }
    return GWGPU_OK;
}

int gwgpu_server_wait(gwgpu_server* s, long long id, double timeout_ms, gwgpu_result* out)
{
    if (!s) return fail(GWGPU_ERR_INVALID, "null server");
    const int rc = s->impl->wait(id, timeout_ms, out);
    if (rc < 0) return fail(GWGPU_ERR_INVALID, "unknown request id");
    if (rc > 0) return fail(GWGPU_ERR_TIMEOUT, "request not finished");
    return GWGPU_OK;
}

int gwgpu_server_poll(gwgpu_server* s, long long id, int* done)
{
    if (!s || !done) return fail(GWGPU_ERR_INVALID, "null argument");
    if (s->impl->poll(id, done) < 0) return fail(GWGPU_ERR_INVALID, "unknown request id");
    return GWGPU_OK;
}

int gwgpu_server_get_stats(gwgpu_server* s, gwgpu_server_stats* out)
{
    if (!s || !out) return fail(GWGPU_ERR_INVALID, "null argument");
    s->impl->stats(out);
    return GWGPU_OK;
}

double gwgpu_server_estimate(gwgpu_server* s, const gwgpu_request* r)
{
    if (!s || !r || r->n < 1 || r->p < 1) return 0.0;
    return s->impl->estimate(*r);
}

double gwgpu_estimate_bytes(int n, int p, int geographic, int precision, int adaptive)
{
    if (n < 1 || p < 1) return 0.0;
    return (double)gwgpu::Engine::estimateBytes(n, p, geographic != 0, precision == GWGPU_MIXED, adaptive != 0, -1);
}

int gwgpu_admit_slot(double budget, int slots, const double* reserved, const int* busy, double estimate)
{
    if (slots < 1 || !reserved || !busy) return -1;
    return gwgpu::admit_slot(budget, slots, reserved, busy, estimate);
}

}  // extern "C"
