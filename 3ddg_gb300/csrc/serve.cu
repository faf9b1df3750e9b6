// Serving form (dg_serve_*): a request loop that admits solves by an HBM
// budget, keeps their state resident on the device and batches their RK steps
// with every other in-flight solve (continuous batching): a request that
// arrives while others run joins the batch at the next step boundary as soon
// as its memory fits, and leaves it when its own step count is reached.
//
// Time is the host's monotonic clock in seconds since dg_serve_create; a
// request's arrival time is given by the caller (an open-loop trace), and its
// latency is completion time minus arrival time.
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
#include <vector>

#include "batch_internal.h"
#include "dg3d.h"
#include "solver_internal.h"

namespace dg {

struct Server {
    struct Req {
        long long id = 0;
        dg_params p{};
        double dt = 0.0;
        int steps = 0;
        size_t bytes = 0;
        double t_arrival = 0.0, t_admit = -1.0, t_done = -1.0;
        int remaining = 0;
        std::vector<double> rho, vel;  // result (when kept)
        int dims[3] = {0, 0, 0};
        // host preparation by the worker thread (fields guarded by mu)
        std::unique_ptr<Batch::Prepared> prep;
        bool prep_done = false;
        int prep_rc = 0;
        std::string prep_err;
        bool failed = false;  // preparation failed; never admitted
        PinnedPool::Block* result = nullptr;  // result copy in flight
    };
    // One tick's device work: its RK steps between two timing events, then
    // the retirements enqueued behind them (a third event).
    struct TickRec {
        cudaEvent_t start = nullptr, end = nullptr, post = nullptr;
        int k = 0;
        std::vector<Req*> done;
    };

    Batch batch;
    size_t budget = 0, in_use = 0;
    bool keep_results = false;
    // Requests by id, inserted by submit under mu (map nodes never move, so
    // the loop keeps plain pointers to them).  The fields a reader of results
    // or statistics sees (times, results, counters) are written under mu.
    std::map<long long, Req> reqs;
    std::deque<Req*> pending;        // loop thread: submitted, not yet admitted (arrival order)
    std::vector<Req*> inflight;      // loop thread: batch index -> request
    std::deque<TickRec> outstanding; // ticks enqueued, not yet seen complete
    std::vector<cudaEvent_t> timing_events, plain_events;
    long long next_id = 1;           // under mu
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    cudaEvent_t base_ev = nullptr;   // host time t_base on the device timeline
    double t_base = 0.0;
    long long ticks = 0;
    double inflight_sum = 0.0;
    double step_s = 0.0;   // running estimate of the device time of one batch step
    double busy_s = 0.0;   // device time in RK steps
    double work = 0.0;     // DOF-stage updates enqueued
    static constexpr int kMaxStepsPerTick = 64;
    static constexpr int kDepth = 2;          // ticks the host may run ahead of the device
    static constexpr int kPrepareAhead = 64;  // requests prepared ahead of admission

    // worker thread: builds arriving requests' meshes ahead of admission
    std::mutex mu;
    std::condition_variable cv_work, cv_ready;
    std::deque<Req*> to_prepare;  // arrival order
    std::vector<Req*> incoming;   // submitted from any thread, not yet seen by the loop
    int prepared_ahead = 0;
    bool stop = false;
    std::thread worker;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    int init(size_t budget_bytes, bool keep)
    {
        budget = budget_bytes;
        keep_results = keep;
        int rc = batch.init(64);
        if (rc) return rc;
        cudaError_t e = cudaEventCreate(&base_ev);
        if (e == cudaSuccess) e = cudaStreamSynchronize(batch.stream);
        if (e == cudaSuccess) e = cudaEventRecord(base_ev, batch.stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(base_ev);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("dg_serve_create: ") + cudaGetErrorString(e));
        t_base = now();
        worker = std::thread([this]() { work_loop(); });
        return DG_OK;
    }

    void work_loop()
    {
        cudaSetDevice(batch.device);
        for (;;) {
            Req* r = nullptr;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv_work.wait(lock, [&] { return stop || (!to_prepare.empty() && prepared_ahead < kPrepareAhead); });
                if (stop) return;
                r = to_prepare.front();
                to_prepare.pop_front();
                prepared_ahead++;
            }
            auto pr = std::make_unique<Batch::Prepared>();
            const int rc = batch.prepare(r->p, r->dt, r->steps, nullptr, nullptr, *pr);
            const std::string err = rc ? dg_last_error() : "";
            {
                std::lock_guard<std::mutex> lock(mu);
                r->prep = std::move(pr);
                r->prep_rc = rc;
                r->prep_err = err;
                r->prep_done = true;
            }
            cv_ready.notify_all();
        }
    }

    ~Server()
    {
        {
            std::lock_guard<std::mutex> lock(mu);
            stop = true;
        }
        cv_work.notify_all();
        if (worker.joinable()) worker.join();
        if (batch.stream) cudaStreamSynchronize(batch.stream);
        for (auto& kv : reqs) {
            kv.second.prep.reset();
            if (kv.second.result) batch.pinned.release_now(kv.second.result);
        }
        for (TickRec& t : outstanding) recycle(t);
        for (cudaEvent_t e : timing_events) cudaEventDestroy(e);
        for (cudaEvent_t e : plain_events) cudaEventDestroy(e);
        if (base_ev) cudaEventDestroy(base_ev);
    }

    cudaEvent_t take_event(bool timing)
    {
        std::vector<cudaEvent_t>& v = timing ? timing_events : plain_events;
        if (!v.empty()) {
            cudaEvent_t e = v.back();
            v.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, timing ? cudaEventDefault : cudaEventDisableTiming);
        return e;
    }

    void recycle(TickRec& t)
    {
        if (t.start) timing_events.push_back(t.start);
        if (t.end) timing_events.push_back(t.end);
        if (t.post) plain_events.push_back(t.post);
        t.start = t.end = t.post = nullptr;
    }

    // Any thread: the request goes to the worker's preparation queue and to
    // the incoming queue, which the loop drains at its next iteration.
    int submit(const dg_params& p, double dt, int steps, double t_arrival, long long* id)
    {
        std::string err = Batch::validate(p);
        if (!err.empty()) return fail(DG_ERR_INVALID, err);
        if (!(dt > 0.0) || steps < 1) return fail(DG_ERR_INVALID, "dg_serve_submit: dt must be > 0 and steps >= 1");
        Req r;
        r.p = p;
        r.p.precision = DG_PRECISION_FP32;
        r.dt = dt;
        r.steps = steps;
        r.remaining = steps;
        r.bytes = batch_problem_bytes(p);
        if (r.bytes > budget)
            return fail(DG_ERR_NOMEM, "dg_serve_submit: request needs " + std::to_string(r.bytes) +
                                          " bytes, more than the whole HBM budget " + std::to_string(budget));
        r.t_arrival = t_arrival < 0.0 ? now() : t_arrival;
        const double ta = r.t_arrival;
        {
            std::lock_guard<std::mutex> lock(mu);
            r.id = next_id++;
            if (id) *id = r.id;
            const long long rid = r.id;
            Req& slot = reqs[rid];
            slot = std::move(r);
            Req* rp = &slot;
            // the preparation queue stays sorted by arrival time
            auto jt = to_prepare.begin();
            while (jt != to_prepare.end() && (*jt)->t_arrival <= ta) ++jt;
            to_prepare.insert(jt, rp);
            incoming.push_back(rp);
        }
        cv_work.notify_one();
        return DG_OK;
    }

    // Loop thread: move submitted requests into pending, sorted by arrival.
    void drain_incoming()
    {
        std::vector<Req*> in;
        {
            std::lock_guard<std::mutex> lock(mu);
            in.swap(incoming);
        }
        for (Req* r : in) {
            auto it = pending.begin();
            while (it != pending.end() && (*it)->t_arrival <= r->t_arrival) ++it;
            pending.insert(it, r);
        }
    }

    bool has_incoming()
    {
        std::lock_guard<std::mutex> lock(mu);
        return !incoming.empty();
    }

    // Admit arrived, prepared requests in arrival order while their memory
    // fits; each admission is stream-ordered device work only.
    int admit(double t)
    {
        while (!pending.empty()) {
            Req& r = *pending.front();
            if (r.t_arrival > t) break;
            if (in_use + r.bytes > budget) break;  // FIFO: later requests wait behind it
            std::unique_ptr<Batch::Prepared> pr;
            {
                std::lock_guard<std::mutex> lock(mu);
                if (!r.prep_done) break;
                pr = std::move(r.prep);
                prepared_ahead--;
                if (r.prep_rc) {
                    // its preparation failed: set it aside (dg_serve_result
                    // reports the error) and go on with the others
                    r.failed = true;
                    pending.pop_front();
                    continue;
                }
            }
            cv_work.notify_one();
            int idx = -1;
            int rc = pr ? batch.commit(*pr, &idx) : fail(DG_ERR_STATE, "serve: request has no preparation");
            if (rc) {
                // keep the prepared request for a later attempt (the error
                // stands for this call)
                std::lock_guard<std::mutex> lock(mu);
                r.prep = std::move(pr);
                prepared_ahead++;
                return rc;
            }
            in_use += r.bytes;
            {
                std::lock_guard<std::mutex> lock(mu);
                r.t_admit = now();
            }
            inflight.push_back(&r);
            pending.pop_front();
        }
        return DG_OK;
    }

    bool prepared(const Req& r)
    {
        std::lock_guard<std::mutex> lock(mu);
        return r.prep_done;
    }

    // Steps the next tick may run without delaying a retirement or the
    // admission of the next arrival: up to the first in-flight solve's end,
    // and only as many steps as fit before the next pending arrival.
    int steps_this_tick(double t)
    {
        int k = kMaxStepsPerTick;
        for (const Req* r : inflight) k = std::min(k, r->remaining);
        if (!pending.empty()) {
            const Req& f = *pending.front();
            const double wait = f.t_arrival - t;
            if (wait <= 0.0) {
                // arrived: waiting for memory (freed by the next retirement)
                // or for its preparation (admit as soon as it is ready)
                if (in_use + f.bytes <= budget) k = 1;
            } else if (step_s > 0.0) {
                k = std::min(k, std::max(1, (int)(wait / step_s)));
            } else {
                k = 1;
            }
        }
        return std::max(1, k);
    }

    // Completion of an enqueued tick: stamps its retired requests with the
    // device time their last step ended (on the host clock) and collects
    // their results.
    int finish(TickRec& t, bool block, bool* done)
    {
        cudaError_t e = block ? cudaEventSynchronize(t.post) : cudaEventQuery(t.post);
        if (e == cudaErrorNotReady) {
            (void)cudaGetLastError();
            *done = false;
            return DG_OK;
        }
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("serve: ") + cudaGetErrorString(e));
        *done = true;
        float ms_end = 0.f, ms_run = 0.f;
        e = cudaEventElapsedTime(&ms_end, base_ev, t.end);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_run, t.start, t.end);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaEventElapsedTime: ") + cudaGetErrorString(e));
        const double t_end = t_base + ms_end * 1e-3;
        const double per = ms_run * 1e-3 / t.k;
        step_s = step_s > 0.0 ? 0.8 * step_s + 0.2 * per : per;
        std::lock_guard<std::mutex> lock(mu);
        busy_s += ms_run * 1e-3;
        for (Req* rp : t.done) {
            Req& r = *rp;
            r.t_done = t_end;
            if (r.result) {
                const size_t g = (size_t)r.dims[0] * r.dims[1] * r.dims[2];
                const double* src = (const double*)r.result->ptr;
                r.rho.assign(src, src + g);
                r.vel.assign(src + g, src + 4 * g);
                batch.pinned.release_now(r.result);
                r.result = nullptr;
            }
        }
        recycle(t);
        return DG_OK;
    }

    int collect(bool block_all)
    {
        while (!outstanding.empty()) {
            bool done = false;
            int rc = finish(outstanding.front(), block_all || (int)outstanding.size() > kDepth, &done);
            if (rc) return rc;
            if (!done) break;
            outstanding.pop_front();
        }
        return DG_OK;
    }

    // One iteration: collect finished ticks, admit, enqueue the tick's steps
    // for every in-flight solve (one graph replay each) and the retirement of
    // the solves they complete (result copy, memory back to the pool), with no
    // host synchronisation; the host waits only to stay at most kDepth ticks
    // ahead of the device, or to drain when nothing is in flight.
    int tick(int* n_inflight)
    {
        drain_incoming();
        int rc = collect(false);
        if (rc) return rc;
        rc = admit(now());
        if (rc) return rc;
        if (!inflight.empty()) {
            const int k = steps_this_tick(now());
            TickRec t;
            t.k = k;
            t.start = take_event(true);
            t.end = take_event(true);
            t.post = take_event(false);
            cudaStream_t st = batch.stream;
            cudaError_t e = cudaEventRecord(t.start, st);
            if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
            rc = batch.step(k);
            if (rc) return rc;
            e = cudaEventRecord(t.end, st);
            if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
            double w = 0.0;
            for (size_t i = 0; i < inflight.size(); i++) {
                const Batch::Entry& E = batch.probs[i];
                w += 4.0 * E.n_elem * E.K * E.K * E.K * 3.0 * k;
                inflight[i]->remaining -= k;
            }
            {
                std::lock_guard<std::mutex> lock(mu);
                work += w;
                ticks += k;
                inflight_sum += (double)inflight.size() * k;
            }
            for (int i = (int)inflight.size() - 1; i >= 0; i--) {
                Req& r = *inflight[i];
                if (r.remaining > 0) continue;
                const Batch::Entry& E = batch.probs[i];
                for (int a = 0; a < 3; a++) r.dims[a] = E.dims[a];
                if (keep_results) {
                    const size_t g = (size_t)E.dims[0] * E.dims[1] * E.dims[2];
                    std::string err;
                    r.result = batch.pinned.acquire(4 * g * sizeof(double), err);
                    if (!r.result) return fail(DG_ERR_CUDA, "serve: " + err);
                    rc = batch.enqueue_state_copy(i, r.steps, r.result);
                    if (rc) return rc;
                }
                rc = batch.remove(i);
                if (rc) return rc;
                in_use -= r.bytes;
                t.done.push_back(&r);
                inflight.erase(inflight.begin() + i);
            }
            e = cudaEventRecord(t.post, st);
            if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
            outstanding.push_back(std::move(t));
        }
        rc = collect(inflight.empty());
        if (rc) return rc;
        if (n_inflight) *n_inflight = (int)inflight.size();
        return DG_OK;
    }

    int run(double max_seconds)
    {
        const double t_end = now() + (max_seconds > 0 ? max_seconds : 1e300);
        drain_incoming();
        while (!pending.empty() || !inflight.empty() || !outstanding.empty() || has_incoming()) {
            if (now() > t_end) return fail(DG_ERR_STATE, "dg_serve_run: time limit reached");
            drain_incoming();
            if (inflight.empty() && !pending.empty()) {
                Req& f = *pending.front();
                const double wait = f.t_arrival - now();
                if (wait > 0) {
                    std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
                } else if (!prepared(f)) {
                    std::unique_lock<std::mutex> lock(mu);
                    cv_ready.wait_for(lock, std::chrono::milliseconds(1), [&] { return f.prep_done; });
                }
            }
            int n = 0;
            int rc = tick(&n);
            if (rc) return rc;
        }
        return DG_OK;
    }
};

}  // namespace dg

struct dg_server {
    dg::Server s;
};

extern "C" {

int dg_serve_create(size_t hbm_budget_bytes, int keep_results, dg_server** out)
{
    if (!out || hbm_budget_bytes == 0) return dg::fail(DG_ERR_INVALID, "dg_serve_create: bad argument");
    *out = nullptr;
    dg_server* h = new (std::nothrow) dg_server;
    if (!h) return dg::fail(DG_ERR_NOMEM, "dg_serve_create: host allocation failed");
    int rc = h->s.init(hbm_budget_bytes, keep_results != 0);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return DG_OK;
}

int dg_serve_destroy(dg_server* s)
{
    delete s;
    return DG_OK;
}

double dg_serve_clock(const dg_server* s) { return s ? s->s.now() : 0.0; }

int dg_serve_submit(dg_server* s, const dg_params* p, double dt, int steps, double arrival_time, long long* id)
{
    if (!s || !p) return dg::fail(DG_ERR_INVALID, "dg_serve_submit: null argument");
    return s->s.submit(*p, dt, steps, arrival_time, id);
}

int dg_serve_tick(dg_server* s, int* n_inflight)
{
    if (!s) return dg::fail(DG_ERR_INVALID, "dg_serve_tick: null handle");
    return s->s.tick(n_inflight);
}

int dg_serve_run(dg_server* s, double max_seconds)
{
    if (!s) return dg::fail(DG_ERR_INVALID, "dg_serve_run: null handle");
    return s->s.run(max_seconds);
}

int dg_serve_result(dg_server* s, long long id, double* t_arrival, double* t_admit, double* t_done, double* drho,
                    double* vel)
{
    if (!s) return dg::fail(DG_ERR_INVALID, "dg_serve_result: null handle");
    std::lock_guard<std::mutex> lock(s->s.mu);
    auto it = s->s.reqs.find(id);
    if (it == s->s.reqs.end()) return dg::fail(DG_ERR_INVALID, "dg_serve_result: unknown request");
    const dg::Server::Req& r = it->second;
    if (r.failed) return dg::fail(r.prep_rc, "dg_serve_result: request failed: " + r.prep_err);
    if (t_arrival) *t_arrival = r.t_arrival;
    if (t_admit) *t_admit = r.t_admit;
    if (t_done) *t_done = r.t_done;
    if (drho || vel) {
        if (r.t_done < 0.0) return dg::fail(DG_ERR_STATE, "dg_serve_result: request not finished");
        if (!s->s.keep_results) return dg::fail(DG_ERR_STATE, "dg_serve_result: server does not keep results");
        if (drho) std::memcpy(drho, r.rho.data(), r.rho.size() * sizeof(double));
        if (vel) std::memcpy(vel, r.vel.data(), r.vel.size() * sizeof(double));
    }
    return DG_OK;
}

int dg_serve_stats(dg_server* s, int* completed, double* p50, double* p99, double* solves_per_s,
                   double* mean_inflight)
{
    if (!s) return dg::fail(DG_ERR_INVALID, "dg_serve_stats: null handle");
    std::lock_guard<std::mutex> lock(s->s.mu);
    std::vector<double> lat;
    double first = 1e300, last = 0.0;
    for (const auto& kv : s->s.reqs) {
        const dg::Server::Req& r = kv.second;
        if (r.t_done < 0.0) continue;
        lat.push_back(r.t_done - r.t_arrival);
        first = std::min(first, r.t_arrival);
        last = std::max(last, r.t_done);
    }
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
        if (lat.empty()) return 0.0;
        const double pos = q * (lat.size() - 1);
        const size_t lo = (size_t)std::floor(pos), hi = std::min(lat.size() - 1, lo + 1);
        return lat[lo] + (pos - lo) * (lat[hi] - lat[lo]);
    };
    if (completed) *completed = (int)lat.size();
    if (p50) *p50 = pct(0.50);
    if (p99) *p99 = pct(0.99);
    if (solves_per_s) *solves_per_s = lat.empty() ? 0.0 : lat.size() / std::max(1e-9, last - first);
    if (mean_inflight) *mean_inflight = s->s.ticks ? s->s.inflight_sum / s->s.ticks : 0.0;
    return DG_OK;
}

int dg_serve_utilization(dg_server* s, double* gpu_busy_s, double* span_s, double* dof_stage_updates)
{
    if (!s) return dg::fail(DG_ERR_INVALID, "dg_serve_utilization: null handle");
    std::lock_guard<std::mutex> lock(s->s.mu);
    double first = 1e300, last = 0.0;
    for (const auto& kv : s->s.reqs) {
        const dg::Server::Req& r = kv.second;
        if (r.t_done < 0.0) continue;
        first = std::min(first, r.t_arrival);
        last = std::max(last, r.t_done);
    }
    if (gpu_busy_s) *gpu_busy_s = s->s.busy_s;
    if (span_s) *span_s = last > first ? last - first : 0.0;
    if (dof_stage_updates) *dof_stage_updates = s->s.work;
    return DG_OK;
}

}  // extern "C"
