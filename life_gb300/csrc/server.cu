// Serving: a request loop that solves LIFE cases as they arrive.
//
// life_server_submit queues a case (params, bodies, step count). A server
// thread admits queued requests in arrival order while their estimated device
// footprint fits the HBM budget, creates their state on the device, and steps
// every admitted request together: the active set is one batch (batch.cu) per
// population storage form, advanced in rounds of at most steps_per_round
// steps and never past the nearest request's end. When a request finishes,
// or a new one is admitted, the active set is regrouped before the next
// round, so requests that arrive while others run join them on the device
// (continuous batching). A finished request keeps its state on the device
// until the client takes the case or releases it; that state counts against
// the budget until then.
//
// Each request computes exactly what it computes alone: inside a batch a case
// runs the same kernels with the same arguments in the same order, and the
// round boundaries only split its steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/life_gb300.h"
#include "life_internal.h"

using namespace life;

namespace life {
int batch_wrap(const std::vector<LifeCase*>& cases, LifeBatch** out);
void batch_free(LifeBatch* b);
int batch_steps(LifeBatch* b, int nsteps);
int batch_failed_case(LifeBatch* b, int* code);
}  // namespace life

namespace {

struct Request {
    int64_t id = 0;
    LifeCaseParams p{};
    std::vector<LifeBodyDesc> bodies;
    int steps = 0, done = 0;
    int state = LIFE_REQ_QUEUED;
    int error = 0;
    std::string msg;
    double submit_s = 0, start_s = 0, done_s = 0;
    size_t estimate = 0, bytes = 0;
    LifeCase* c = nullptr;
};

// Device bytes of a case before it exists: both population buffers, the
// per-row side buffers, the dense IBM force and scratch when bodies are
// present, and a per-body allowance for markers, supports and FEM state.
size_t estimate_bytes(const LifeCaseParams& p, int n_bodies) {
    const size_t elem = p.precision == LIFE_PREC_F64 ? 8 : (p.precision == LIFE_PREC_F32 ? 4 : 2);
    const size_t pitch = ((size_t)p.Nx + 63) / 64 * 64;
    const size_t S = pitch * (size_t)p.Ny;
    size_t b = 2 * 9 * elem * S + 24 * 8 * (size_t)p.Ny + (1 << 16);
    if (n_bodies > 0) b += 20 * S + (size_t)n_bodies * (1 << 20);
    return b;
}

}  // namespace

struct LifeServer {
    LifeServerConfig cfg{};
    int device = 0;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<int64_t> queue;
    std::map<int64_t, Request> reqs;
    std::vector<int64_t> active;
    int creating = 0;  // admitted, device state being created
    bool stop = false;
    int64_t next_id = 1;
    LifeServerStats st{};
    std::chrono::steady_clock::time_point t0;
    double busy_since = -1.0;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    void loop();
};

void LifeServer::loop() {
    cudaSetDevice(device);
    std::vector<std::pair<int, LifeBatch*>> groups;  // (storage form, batch)
    std::vector<int64_t> grouped;                     // active set the groups were built for
    auto free_groups = [&]() {
        for (auto& g : groups) batch_free(g.second);
        groups.clear();
        grouped.clear();
    };
    for (;;) {
        std::vector<int64_t> to_create;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (stop) {  // running requests are abandoned; destroy frees them
                lk.unlock();
                free_groups();
                return;
            }
            for (;;) {
                while (!queue.empty() && (cfg.max_active <= 0 || (int)(active.size() + to_create.size()) < cfg.max_active)) {
                    Request& r = reqs[queue.front()];
                    if (st.bytes_in_use + r.estimate > cfg.hbm_budget && !(active.empty() && to_create.empty() &&
                                                                           st.bytes_in_use == 0))
                        break;
                    queue.pop_front();
                    st.bytes_in_use += r.estimate;
                    to_create.push_back(r.id);
                    creating++;
                }
                if (!to_create.empty() || !active.empty()) break;
                if (stop) {
                    lk.unlock();
                    free_groups();
                    return;
                }
                if (busy_since >= 0) {
                    st.busy_s += now() - busy_since;
                    busy_since = -1.0;
                }
                cv.wait(lk);
            }
            if (busy_since < 0) busy_since = now();
            st.queued = (int32_t)queue.size();
        }
        // create admitted requests' device state (outside the lock)
        for (int64_t id : to_create) {
            LifeCaseParams p;
            std::vector<LifeBodyDesc> bodies;
            {
                std::lock_guard<std::mutex> lk(mu);
                p = reqs[id].p;
                bodies = reqs[id].bodies;
            }
            LifeCase* c = nullptr;
            int rc = life_case_create(&p, bodies.data(), (int32_t)bodies.size(), &c);
            std::string msg = rc ? life_last_error() : "";
            std::lock_guard<std::mutex> lk(mu);
            Request& r = reqs[id];
            st.bytes_in_use -= r.estimate;
            creating--;
            if (rc) {
                r.state = LIFE_REQ_FAILED;
                r.error = rc;
                r.msg = msg;
                r.done_s = now();
                st.failed++;
                cv_done.notify_all();
                continue;
            }
            r.c = c;
            r.bytes = c->dev_bytes;
            st.bytes_in_use += r.bytes;
            st.bytes_peak = std::max(st.bytes_peak, st.bytes_in_use);
            r.state = LIFE_REQ_RUNNING;
            r.start_s = now();
            st.admitted++;
            active.push_back(id);
        }
        if (active.empty()) continue;
        // regroup when the active set changed
        if (grouped != active) {
            free_groups();
            std::map<int, std::vector<LifeCase*>> byprec;
            {
                std::lock_guard<std::mutex> lk(mu);
                for (int64_t id : active) byprec[reqs[id].p.precision].push_back(reqs[id].c);
            }
            bool ok = true;
            std::string err;
            for (auto& kv : byprec) {
                LifeBatch* b = nullptr;
                if (batch_wrap(kv.second, &b)) {
                    ok = false;
                    err = life_last_error();
                    break;
                }
                groups.push_back({kv.first, b});
            }
            if (!ok) {
                free_groups();
                std::lock_guard<std::mutex> lk(mu);
                for (int64_t id : active) {
                    Request& r = reqs[id];
                    r.state = LIFE_REQ_FAILED;
                    r.error = LIFE_ERR_CUDA;
                    r.msg = err;
                    r.done_s = now();
                    st.failed++;
                }
                active.clear();
                cv_done.notify_all();
                continue;
            }
            grouped = active;
            st.regroups++;
        }
        int chunk = cfg.steps_per_round > 0 ? cfg.steps_per_round : 200;
        long long sites = 0;
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int64_t id : active) {
                const Request& r = reqs[id];
                chunk = std::min(chunk, r.steps - r.done);
                sites += (long long)r.p.Nx * r.p.Ny;
            }
        }
        // one round: every group advances `chunk` steps
        std::vector<std::pair<int64_t, std::pair<int, std::string>>> failed;
        bool all_failed = false;
        std::string all_msg;
        int all_code = 0;
        if (chunk > 0) {
            for (auto& g : groups) {
                int rc = batch_steps(g.second, chunk);
                if (!rc) continue;
                int code = 0;
                const int k = batch_failed_case(g.second, &code);
                if (k < 0) {
                    all_failed = true;
                    all_code = rc;
                    all_msg = life_last_error();
                    continue;
                }
                // device-status failures: every case of the group that raised one
                std::lock_guard<std::mutex> lk(mu);
                for (int64_t id : active) {
                    Request& r = reqs[id];
                    if (r.c && r.c->status_code) failed.push_back({id, {r.c->status_code, r.c->status_msg}});
                }
            }
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            st.rounds++;
            st.site_steps += (double)sites * chunk;
            std::vector<int64_t> keep;
            for (int64_t id : active) {
                Request& r = reqs[id];
                r.done += chunk;
                bool fail = all_failed;
                int code = all_code;
                std::string msg = all_msg;
                for (auto& f : failed)
                    if (f.first == id) {
                        fail = true;
                        code = f.second.first;
                        msg = f.second.second;
                    }
                if (fail) {
                    r.state = LIFE_REQ_FAILED;
                    r.error = code;
                    r.msg = msg;
                    r.done_s = now();
                    st.failed++;
                } else if (r.done >= r.steps) {
                    r.state = LIFE_REQ_DONE;
                    r.done_s = now();
                    st.completed++;
                } else {
                    keep.push_back(id);
                }
            }
            if (keep.size() != active.size()) cv_done.notify_all();
            active.swap(keep);
            st.active = (int32_t)active.size();
        }
        if (grouped != active) free_groups();
    }
}

extern "C" int life_server_create(const LifeServerConfig* cfg, LifeServer** out) {
    if (!cfg || !out) return set_error(LIFE_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (cfg->hbm_budget == 0) return set_error(LIFE_ERR_INVALID, "hbm_budget must be positive");
    LifeServer* s = new LifeServer();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    s->t0 = std::chrono::steady_clock::now();
    s->th = std::thread([s]() { s->loop(); });
    *out = s;
    return LIFE_OK;
}

extern "C" int life_server_submit(LifeServer* s, const LifeCaseParams* p, const LifeBodyDesc* bodies,
                                  int32_t n_bodies, int32_t nsteps, int64_t* id) {
    if (!s || !p || !id || nsteps <= 0 || n_bodies < 0 || (n_bodies > 0 && !bodies))
        return set_error(LIFE_ERR_INVALID, "bad request");
    Request r;
    r.p = *p;
    r.bodies.assign(bodies, bodies + n_bodies);
    r.steps = nsteps;
    r.estimate = estimate_bytes(*p, n_bodies);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_error(LIFE_ERR_BUSY, "server is shutting down");
    r.id = s->next_id++;
    r.submit_s = s->now();
    *id = r.id;
    s->queue.push_back(r.id);
    s->reqs[r.id] = std::move(r);
    s->st.submitted++;
    s->st.queued = (int32_t)s->queue.size();
    s->cv.notify_all();
    return LIFE_OK;
}

extern "C" int life_server_query(LifeServer* s, int64_t id, LifeRequestInfo* info) {
    if (!s || !info) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(LIFE_ERR_INVALID, "no such request");
    const Request& r = it->second;
    LifeRequestInfo I{};
    I.state = r.state;
    I.error = r.error;
    I.steps = r.steps;
    I.steps_done = std::min(r.done, r.steps);
    I.submit_s = r.submit_s;
    I.start_s = r.start_s;
    I.done_s = r.done_s;
    I.device_bytes = r.bytes;
    I.sites = (int64_t)r.p.Nx * r.p.Ny;
    *info = I;
    if (r.state == LIFE_REQ_FAILED) set_error(r.error, r.msg);
    return LIFE_OK;
}

extern "C" int life_server_wait(LifeServer* s, int64_t id, double timeout_s) {
    if (!s) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&]() {
        auto it = s->reqs.find(id);
        return it == s->reqs.end() || it->second.state == LIFE_REQ_DONE || it->second.state == LIFE_REQ_FAILED;
    };
    const auto limit = std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s);
    if (!s->cv_done.wait_for(lk, limit, done)) return set_error(LIFE_ERR_TIMEOUT, "request not finished");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(LIFE_ERR_INVALID, "no such request");
    if (it->second.state == LIFE_REQ_FAILED) return set_error(it->second.error, it->second.msg);
    return LIFE_OK;
}

extern "C" int life_server_take(LifeServer* s, int64_t id, LifeCase** out) {
    if (!s || !out) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second.state != LIFE_REQ_DONE || !it->second.c)
        return set_error(LIFE_ERR_BUSY, "request not finished or already taken");
    *out = it->second.c;
    it->second.c = nullptr;
    s->st.bytes_in_use -= it->second.bytes;
    s->cv.notify_all();
    return LIFE_OK;
}

extern "C" int life_server_release(LifeServer* s, int64_t id) {
    if (!s) return set_error(LIFE_ERR_INVALID, "NULL argument");
    LifeCase* c = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) return set_error(LIFE_ERR_INVALID, "no such request");
        Request& r = it->second;
        if (r.state != LIFE_REQ_DONE && r.state != LIFE_REQ_FAILED)
            return set_error(LIFE_ERR_BUSY, "request still queued or running");
        c = r.c;
        if (c) s->st.bytes_in_use -= r.bytes;
        s->reqs.erase(it);
    }
    if (c) life_case_destroy(c);
    s->cv.notify_all();
    return LIFE_OK;
}

extern "C" int life_server_stats(LifeServer* s, LifeServerStats* out) {
    if (!s || !out) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    LifeServerStats S = s->st;
    S.clock_s = s->now();
    if (s->busy_since >= 0) S.busy_s += S.clock_s - s->busy_since;
    *out = S;
    return LIFE_OK;
}

extern "C" int life_server_drain(LifeServer* s, double timeout_s) {
    if (!s) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto limit = std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s);
    if (!s->cv_done.wait_for(lk, limit,
                             [&]() { return s->queue.empty() && s->active.empty() && s->creating == 0; }))
        return set_error(LIFE_ERR_TIMEOUT, "requests still queued or running");
    return LIFE_OK;
}

extern "C" int life_server_destroy(LifeServer* s) {
    if (!s) return LIFE_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->queue.clear();
        s->cv.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    for (auto& kv : s->reqs)
        if (kv.second.c) life_case_destroy(kv.second.c);
    delete s;
    return LIFE_OK;
}
