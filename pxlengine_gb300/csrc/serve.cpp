// Serving form: a continuous-batching request loop over the batched substep engine.
//
// Each request is one liquid simulation (a fluid description, seed, fps, options) and a number of
// substeps. A tick
//   1. retires active requests that reached their substep count: their final particles are read
//      into host memory and their device memory is released;
//   2. admits queued requests in arrival order while the sum of the estimated device footprints
//      (pxf_estimate_bytes) stays within the HBM budget and a slot is free;
//   3. advances every active request by `substeps_per_tick` substeps in ONE batched launch
//      sequence (one CUDA graph launch per substep for all of them), timed with CUDA events.
// Requests that arrive while others run join the next tick's batch, so their work overlaps on
// the device. Every reduction of the substep is per simulation, so a request's result does not
// depend on which other requests shared its batches.
//
// The server uses only the public C ABI (include/pxlflip.h).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "../../include/pxlflip.h"
#include "scene.h"

namespace {

struct Request {
    uint64_t id = 0;
    pxf::FluidCfg cfg;
    uint32_t seed = 0;
    double fps = 24.0;
    pxf_options opts;
    uint32_t total = 0;
    uint32_t done = 0;
    int state = PXF_REQ_QUEUED;
    int error = 0;
    uint64_t bytes = 0;
    uint32_t particles = 0;
    pxf_sim* sim = nullptr;
    std::vector<float> result;
    double submit_s = 0, admit_s = 0, finish_s = 0;
    std::string message;
};

double pct(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * double(v.size() - 1);
    const size_t i = size_t(pos);
    const double f = pos - double(i);
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

struct pxf_server {
    pxf_server_config cfg;
    std::mutex mu;                              // guards everything below except the batch
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    std::deque<uint64_t> queue;
    std::vector<Request*> active;
    uint64_t next_id = 1;
    uint64_t reserved = 0, peak_reserved = 0;
    uint64_t ticks = 0, submitted = 0, admitted = 0, completed = 0, cancelled = 0, rejected = 0;
    double particle_substeps = 0, busy_ms = 0;
    std::vector<double> substep_ms, tick_wall_ms;
    pxf_batch* batch = nullptr;
    std::mutex tick_mu;                         // one tick at a time
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::string err;
    std::thread worker;
    std::atomic<bool> running{false};
    std::condition_variable cv;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    int fail(int code, const std::string& m) {
        err = m;
        return code;
    }
};

namespace {

// Moves a finished or cancelled request's particles to the host and frees its device state.
void release(pxf_server* S, Request* r, bool keep_result) {
    if (!r->sim) return;
    pxf::trace("serve: release request %llu", (unsigned long long)r->id);
    pxf_batch_remove(S->batch, r->sim);
    if (keep_result) {
        r->result.resize(size_t(r->particles) * 8);
        int rc = pxf_read_particles(r->sim, r->result.data(), r->particles);
        if (rc) {
            r->state = PXF_REQ_FAILED;
            r->error = rc;
            r->message = pxf_last_error(r->sim);
            r->result.clear();
        }
    }
    pxf_destroy(r->sim);
    r->sim = nullptr;
    S->reserved -= r->bytes;
}

int tick_impl(pxf_server* S, uint32_t* active_out) {
    std::lock_guard<std::mutex> tl(S->tick_mu);
    const auto w0 = std::chrono::steady_clock::now();
    std::vector<Request*> step_set;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        // 1. retire finished and cancelled requests
        std::vector<Request*> still;
        for (Request* r : S->active) {
            if (r->state == PXF_REQ_CANCELLED || r->state == PXF_REQ_FAILED) {
                release(S, r, false);
            } else if (r->done >= r->total) {
                release(S, r, true);
                if (r->state != PXF_REQ_FAILED) {
                    r->state = PXF_REQ_DONE;
                    S->completed++;
                }
                r->finish_s = S->now();
            } else {
                still.push_back(r);
            }
        }
        S->active.swap(still);
        // 2. admit in arrival order while the budget and the slots allow
        while (!S->queue.empty() && S->active.size() < S->cfg.max_active) {
            Request* r = S->reqs[S->queue.front()].get();
            if (r->state == PXF_REQ_CANCELLED) {
                S->queue.pop_front();
                continue;
            }
            if (S->reserved + r->bytes > S->cfg.hbm_budget_bytes) break;   // head-of-line waits for memory
            S->queue.pop_front();
            pxf_fluid_desc d;
            r->cfg.to_desc(d);
            pxf_sim* sim = nullptr;
            pxf::trace("serve: admit request %llu", (unsigned long long)r->id);
            int rc = pxf_create_ex(&d, r->seed, r->fps, &r->opts, &sim);
            pxf::trace("serve: created rc=%d", rc);
            if (rc == PXF_OK) rc = pxf_batch_add(S->batch, sim);
            if (rc != PXF_OK) {
                r->state = PXF_REQ_FAILED;
                r->error = rc;
                r->message = sim ? pxf_last_error(sim) : pxf_last_error(nullptr);
                if (sim) pxf_destroy(sim);
                r->finish_s = S->now();
                continue;
            }
            r->sim = sim;
            r->particles = pxf_particle_count(sim);
            r->state = PXF_REQ_RUNNING;
            r->admit_s = S->now();
            S->reserved += r->bytes;
            S->peak_reserved = std::max(S->peak_reserved, S->reserved);
            S->admitted++;
            S->active.push_back(r);
        }
        step_set = S->active;
    }
    // 3. one batched substep (or substeps_per_tick) for every active request
    int rc = PXF_OK;
    double ms = 0;
    uint32_t n = S->cfg.substeps_per_tick ? S->cfg.substeps_per_tick : 1;
    if (!step_set.empty()) {
        uint32_t need = n;
        for (Request* r : step_set) need = std::min(need, r->total - r->done);
        if (need == 0) need = 1;
        pxf::trace("serve: step %zu requests", step_set.size());
        rc = pxf_batch_step_timed(S->batch, need, &ms);
        pxf::trace("serve: step rc=%d", rc);
        std::lock_guard<std::mutex> lk(S->mu);
        if (rc != PXF_OK) {
            S->err = pxf_batch_last_error(S->batch);
            for (Request* r : step_set) {
                r->state = PXF_REQ_FAILED;
                r->error = rc;
                r->message = S->err;
            }
        } else {
            for (Request* r : step_set) {
                r->done += need;
                S->particle_substeps += double(r->particles) * need;
            }
            S->busy_ms += ms;
            S->substep_ms.push_back(ms / need);
            S->ticks++;
        }
    }
    const double wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    std::lock_guard<std::mutex> lk(S->mu);
    if (!step_set.empty()) S->tick_wall_ms.push_back(wall);
    if (active_out) *active_out = uint32_t(S->active.size());
    return rc;
}

}  // namespace

extern "C" {

void pxf_server_config_init(pxf_server_config* c) {
    if (!c) return;
    c->hbm_budget_bytes = 150000000000ull;
    c->max_active = 256;
    c->substeps_per_tick = 1;
    c->wait_timeout_s = 600.0;
}

int pxf_server_create(const pxf_server_config* cfg, pxf_server** out) {
    if (!out) return PXF_EINVAL;
    std::unique_ptr<pxf_server> S(new pxf_server());
    if (cfg) S->cfg = *cfg; else pxf_server_config_init(&S->cfg);
    if (S->cfg.max_active == 0) S->cfg.max_active = 1;
    int rc = pxf_batch_create(&S->batch);
    if (rc) return rc;
    *out = S.release();
    return PXF_OK;
}

int pxf_server_submit(pxf_server* S, const pxf_fluid_desc* desc, uint32_t seed, double fps, const pxf_options* opts,
                      uint32_t substeps, uint64_t* id) {
    if (!S || !desc || !id) return PXF_EINVAL;
    std::unique_ptr<Request> r(new Request());
    r->cfg.from_desc(*desc);
    r->seed = seed;
    r->fps = fps;
    if (opts) r->opts = *opts; else pxf_options_init(&r->opts);
    r->opts.wait_timeout_s = S->cfg.wait_timeout_s;
    r->total = substeps;
    std::string msg;
    if (!pxf::validate_fluid(r->cfg, 0, r->opts.lift_grid_limits != 0, msg)) return S->fail(PXF_EINVAL, msg);
    uint64_t bytes = 0;
    int rc = pxf_estimate_bytes(desc, &r->opts, &bytes);
    if (rc) return S->fail(rc, "footprint estimate failed");
    r->bytes = bytes;
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    r->submit_s = S->now();
    *id = r->id;
    S->submitted++;
    if (bytes > S->cfg.hbm_budget_bytes) {
        r->state = PXF_REQ_FAILED;
        r->error = PXF_ENOMEM;
        r->message = "request needs " + std::to_string(bytes) + " bytes, over the HBM budget of " +
                     std::to_string(S->cfg.hbm_budget_bytes);
        r->finish_s = r->submit_s;
        S->rejected++;
        S->err = r->message;
        S->reqs[r->id] = std::move(r);
        return PXF_ENOMEM;
    }
    S->queue.push_back(r->id);
    S->reqs[r->id] = std::move(r);
    S->cv.notify_all();
    return PXF_OK;
}

int pxf_server_cancel(pxf_server* S, uint64_t id) {
    if (!S) return PXF_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return S->fail(PXF_ENOTFOUND, "unknown request");
    Request* r = it->second.get();
    if (r->state == PXF_REQ_QUEUED || r->state == PXF_REQ_RUNNING) {
        r->state = PXF_REQ_CANCELLED;
        r->finish_s = S->now();
        S->cancelled++;
    }
    return PXF_OK;
}

int pxf_server_tick(pxf_server* S, uint32_t* active) {
    if (!S) return PXF_EINVAL;
    return tick_impl(S, active);
}

int pxf_server_status(pxf_server* S, uint64_t id, pxf_request_status* out) {
    if (!S || !out) return PXF_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return S->fail(PXF_ENOTFOUND, "unknown request");
    const Request* r = it->second.get();
    out->state = r->state;
    out->error = r->error;
    out->substeps_done = r->done;
    out->substeps_total = r->total;
    out->particles = r->particles;
    out->device_bytes = r->bytes;
    out->submit_s = r->submit_s;
    out->admit_s = r->admit_s;
    out->finish_s = r->finish_s;
    return PXF_OK;
}

int pxf_server_take_result(pxf_server* S, uint64_t id, float* out, size_t n) {
    if (!S || !out) return PXF_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return S->fail(PXF_ENOTFOUND, "unknown request");
    Request* r = it->second.get();
    if (r->state != PXF_REQ_DONE) return S->fail(PXF_ESTATE, "request has no result (state " + std::to_string(r->state) + ")");
    if (n != r->particles) return S->fail(PXF_EINVAL, "particle count mismatch");
    std::memcpy(out, r->result.data(), r->result.size() * sizeof(float));
    S->reqs.erase(it);
    return PXF_OK;
}

int pxf_server_stats_get(pxf_server* S, pxf_server_stats* o) {
    if (!S || !o) return PXF_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(o, 0, sizeof(*o));
    o->ticks = S->ticks;
    o->submitted = S->submitted;
    o->admitted = S->admitted;
    o->completed = S->completed;
    o->cancelled = S->cancelled;
    o->rejected = S->rejected;
    o->active = uint32_t(S->active.size());
    o->queued = uint32_t(S->queue.size());
    o->reserved_bytes = S->reserved;
    o->peak_reserved_bytes = S->peak_reserved;
    o->particle_substeps = S->particle_substeps;
    o->busy_device_ms = S->busy_ms;
    o->p50_substep_ms = pct(S->substep_ms, 0.50);
    o->p99_substep_ms = pct(S->substep_ms, 0.99);
    o->p50_tick_wall_ms = pct(S->tick_wall_ms, 0.50);
    o->p99_tick_wall_ms = pct(S->tick_wall_ms, 0.99);
    o->uptime_s = S->now();
    return PXF_OK;
}

int pxf_server_start(pxf_server* S) {
    if (!S) return PXF_EINVAL;
    if (S->running.exchange(true)) return PXF_OK;
    S->worker = std::thread([S]() {
        while (S->running.load()) {
            bool work;
            {
                std::unique_lock<std::mutex> lk(S->mu);
                work = !S->queue.empty() || !S->active.empty();
                if (!work) S->cv.wait_for(lk, std::chrono::milliseconds(2));
            }
            if (work) {
                if (tick_impl(S, nullptr) != PXF_OK) std::this_thread::sleep_for(std::chrono::milliseconds(1));
            }
        }
    });
    return PXF_OK;
}

int pxf_server_stop(pxf_server* S) {
    if (!S) return PXF_EINVAL;
    if (S->running.exchange(false)) {
        S->cv.notify_all();
        if (S->worker.joinable()) S->worker.join();
    }
    return PXF_OK;
}

void pxf_server_destroy(pxf_server* S) {
    if (!S) return;
    pxf_server_stop(S);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (Request* r : S->active) release(S, r, false);
        S->active.clear();
    }
    pxf_batch_destroy(S->batch);
    delete S;
}

const char* pxf_server_last_error(const pxf_server* S) { return S ? S->err.c_str() : ""; }

}  // extern "C"
