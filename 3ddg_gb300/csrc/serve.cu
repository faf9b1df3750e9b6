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
#include <cstring>
#include <deque>
#include <map>
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
    };
    Batch batch;
    size_t budget = 0, in_use = 0;
    bool keep_results = false;
    std::map<long long, Req> reqs;
    std::deque<long long> pending;   // submitted, not yet arrived or not yet admitted (arrival order)
    std::vector<long long> inflight; // batch index -> request id
    long long next_id = 1;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    long long ticks = 0;
    double inflight_sum = 0.0;
    double step_s = 0.0;  // running estimate of the wall time of one batch step
    static constexpr int kMaxStepsPerTick = 64;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    int submit(const dg_params& p, double dt, int steps, double t_arrival, long long* id)
    {
        std::string err = Batch::validate(p);
        if (!err.empty()) return fail(DG_ERR_INVALID, err);
        if (!(dt > 0.0) || steps < 1) return fail(DG_ERR_INVALID, "dg_serve_submit: dt must be > 0 and steps >= 1");
        Req r;
        r.id = next_id++;
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
        // keep pending sorted by arrival time
        auto it = pending.begin();
        while (it != pending.end() && reqs[*it].t_arrival <= r.t_arrival) ++it;
        pending.insert(it, r.id);
        if (id) *id = r.id;
        reqs[r.id] = std::move(r);
        return DG_OK;
    }

    // Admit arrived requests in arrival order while their memory fits.
    int admit(double t)
    {
        while (!pending.empty()) {
            Req& r = reqs[pending.front()];
            if (r.t_arrival > t) break;
            if (in_use + r.bytes > budget) break;  // FIFO: later requests wait behind it
            int idx = -1;
            int rc = batch.add(r.p, r.dt, r.steps, nullptr, nullptr, &idx);
            if (rc) return rc;
            in_use += r.bytes;
            r.t_admit = now();
            inflight.push_back(r.id);
            pending.pop_front();
        }
        return DG_OK;
    }

    int retire(double t)
    {
        for (int i = (int)inflight.size() - 1; i >= 0; i--) {
            Req& r = reqs[inflight[i]];
            if (r.remaining > 0) continue;
            if (keep_results) {
                const Batch::Entry& E = batch.probs[i];
                for (int a = 0; a < 3; a++) r.dims[a] = E.dims[a];
                const size_t g = (size_t)E.dims[0] * E.dims[1] * E.dims[2];
                r.rho.resize(g);
                r.vel.resize(3 * g);
                int rc = batch.get_state(i, r.rho.data(), r.vel.data());
                if (rc) return rc;
            }
            r.t_done = t;
            int rc = batch.remove(i);
            if (rc) return rc;
            in_use -= r.bytes;
            inflight.erase(inflight.begin() + i);
        }
        return DG_OK;
    }

    // Steps the next tick may run without delaying a retirement or the
    // admission of the next arrival: up to the first in-flight solve's end,
    // and only as many steps as fit before the next pending arrival.
    int steps_this_tick(double t) const
    {
        int k = kMaxStepsPerTick;
        for (long long id : inflight) k = std::min(k, reqs.at(id).remaining);
        if (!pending.empty()) {
            const double wait = reqs.at(pending.front()).t_arrival - t;
            if (wait <= 0.0) return 1;  // arrived, waiting for memory: retire as soon as possible
            if (step_s > 0.0) k = std::min(k, std::max(1, (int)(wait / step_s)));
            else k = 1;
        }
        return std::max(1, k);
    }

    // One iteration: admit, advance every in-flight solve by the tick's
    // steps (one graph replay each, one host synchronisation), retire.
    int tick(int* n_inflight)
    {
        int rc = admit(now());
        if (rc) return rc;
        if (!inflight.empty()) {
            const double t_start = now();
            const int k = steps_this_tick(t_start);
            rc = batch.step(k);
            if (rc) return rc;
            cudaError_t e = cudaStreamSynchronize(batch.stream);
            if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
            const double per = (now() - t_start) / k;
            step_s = step_s > 0.0 ? 0.8 * step_s + 0.2 * per : per;
            for (long long id : inflight) reqs[id].remaining -= k;
            ticks += k;
            inflight_sum += (double)inflight.size() * k;
            rc = retire(now());
            if (rc) return rc;
        }
        if (n_inflight) *n_inflight = (int)inflight.size();
        return DG_OK;
    }

    int run(double max_seconds)
    {
        const double t_end = now() + (max_seconds > 0 ? max_seconds : 1e300);
        while (!pending.empty() || !inflight.empty()) {
            if (now() > t_end) return fail(DG_ERR_STATE, "dg_serve_run: time limit reached");
            if (inflight.empty() && !pending.empty()) {
                const double wait = reqs[pending.front()].t_arrival - now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
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
    h->s.budget = hbm_budget_bytes;
    h->s.keep_results = keep_results != 0;
    int rc = h->s.batch.init(64);
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
    auto it = s->s.reqs.find(id);
    if (it == s->s.reqs.end()) return dg::fail(DG_ERR_INVALID, "dg_serve_result: unknown request");
    const dg::Server::Req& r = it->second;
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

}  // extern "C"
