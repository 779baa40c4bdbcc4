// server.cpp — request loop for mobility solves with continuous batching on one GPU.
//
// The reference solves one system at a time inside SphereSystem::resolveCollision
// (SRC/SphereSystem.cpp:403-479); this server accepts independent mobility problems as they
// arrive and keeps several of them on the GPU at once:
//   * submit() copies the request (geometry, forces, tolerance) into a FIFO queue and returns at once;
//   * worker threads (one per slot) admit the queue head when a slot is free and its device-memory
//     footprint fits in the budget left by the requests already on the GPU; an admitted request gets
//     its own context on its own non-blocking stream, so its kernels overlap with the other
//     requests' kernels on the device while its Krylov state stays device-resident;
//   * contexts allocate with the stream-ordered allocator, so admitting or retiring a request never
//     synchronizes the device;
//   * each request is solved exactly as it would be alone (its own context, deterministic kernels),
//     so results do not depend on what else is in flight.
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

#include "../../include/smob.h"

namespace smob {
void set_last_error(const char* msg);
smob_status create_context(smob_ctx** out, const smob_geometry* geo, int device, int priority_rank);
}

namespace {

struct Request {
    long long id = 0;
    int n = 0;
    std::vector<double> centers, radii, quats, force, vel;
    std::vector<int> orders;
    bool has_quats = false;
    double viscosity = 1.0, tol = 1e-8;
    size_t bytes = 0;
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = SMOB_OK;
    double t_submit = 0, t_admit = 0, t_done = 0;
    smob_problem_stats stats{};
    std::string error;
};

}  // namespace

struct smob_server {
    smob_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv;       // workers wait for admissible work
    std::condition_variable done_cv;  // waiters wait for completions
    std::deque<long long> queue;
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::vector<std::thread> workers;
    bool stop = false;
    long long next_id = 1;
    double budget = 0, used = 0, peak_used = 0;
    int running = 0, peak_running = 0;
    long long completed = 0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    void worker() {
        for (;;) {
            Request* r = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] {
                    if (stop) return true;
                    if (queue.empty()) return false;
                    const Request* h = reqs[queue.front()].get();
                    return used + double(h->bytes) <= budget || running == 0;
                });
                if (stop) return;
                r = reqs[queue.front()].get();
                queue.pop_front();
                used += double(r->bytes);
                peak_used = std::max(peak_used, used);
                ++running;
                peak_running = std::max(peak_running, running);
                r->state = 1;
                r->t_admit = now();
            }
            run(r);
            {
                std::lock_guard<std::mutex> lk(mu);
                used -= double(r->bytes);
                --running;
                ++completed;
                r->state = 2;
                r->t_done = now();
            }
            cv.notify_all();
            done_cv.notify_all();
        }
    }

    void run(Request* r) {
        smob_geometry g{r->n, r->centers.data(), r->radii.data(), r->has_quats ? r->quats.data() : nullptr,
                        r->orders.data(), nullptr, r->viscosity};
        smob_ctx* ctx = nullptr;
        // stream priority by size: requests with fewer far-field pairs get higher priority, so their
        // kernels are scheduled between the blocks of large requests' long launches
        double pts = 0;
        for (int o : r->orders) pts += double(o + 1) * (2 * o + 2);
        const double pairs = pts * pts;
        const int rank = pairs < 1e9 ? 0 : (pairs < 3e10 ? 1 : 2);
        smob_status s = smob::create_context(&ctx, &g, opts.device, rank);
        if (s == SMOB_OK) {
            smob_solve_opts o{r->tol, opts.restart, opts.max_iters, opts.precision, SMOB_WARM_NONE, opts.inner_tol, 0};
            r->vel.assign(6 * r->n, 0.0);
            s = smob_solve_mob(ctx, r->force.data(), r->vel.data(), nullptr, &o, &r->stats);
        }
        if (s != SMOB_OK) r->error = smob_last_error();
        r->status = s;
        smob_destroy(ctx);
    }
};

namespace {

size_t request_bytes(int n, const int* orders, int restart) {
    size_t M = 0, coef = 0, setsrc = 0;
    int pmax = 1;
    for (int i = 0; i < n; ++i) {
        const int p = orders[i];
        M += size_t(p + 1) * (2 * p + 2);
        coef += size_t(3) * (p + 1) * (p + 2) / 2;
        pmax = std::max(pmax, p);
    }
    setsrc = size_t(2) * 25 * (pmax + 4) * (pmax + 5) / 2;
    const size_t chunks = 16;
    size_t b = 0;
    b += size_t(8) * 3 * M * (restart + 1);  // Krylov basis
    b += size_t(8) * 3 * M * 15;              // solver and staging vectors
    b += size_t(20) * 3 * M * chunks;         // far-field partial sums (FP32 + 2 x FP64)
    b += size_t(160) * M;                     // point data (FP64 + FP32 + float-float)
    b += size_t(12) * 2 * coef;               // coefficients (FP32 + FP64)
    b += size_t(12) * setsrc * size_t(n);     // near-field sets (upper bound: every sphere a source)
    b += size_t(96) * M;                      // coarse equivalent sources: points and strengths of both sets
    b += size_t(700) * M;                     // coarse targets: level slots (9 x (12 + 48) B per point), node
                                              // values, normals and partial sums of both sets
    b += size_t(96) << 20;                    // tables, coarse maps (and their transposes) and small arrays
    return b;
}

}  // namespace

extern "C" {

size_t smob_request_bytes(int n_spheres, const int* orders, int restart) {
    if (n_spheres <= 0 || !orders) return 0;
    return request_bytes(n_spheres, orders, std::max(1, restart));
}

smob_status smob_server_create(smob_server** out, const smob_server_opts* o) {
    if (!out || !o) {
        smob::set_last_error("null argument");
        return SMOB_ERR_ARG;
    }
    if (o->max_slots < 1 || o->restart < 1 || o->max_iters < 1) {
        smob::set_last_error("server options: max_slots, restart and max_iters must be positive");
        return SMOB_ERR_ARG;
    }
    auto* s = new smob_server;
    s->opts = *o;
    s->budget = o->hbm_budget_bytes > 0 ? o->hbm_budget_bytes : 64.0e9;
    for (int i = 0; i < o->max_slots; ++i) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return SMOB_OK;
}

smob_status smob_server_submit(smob_server* s, const smob_geometry* g, const double* force6n, double tol,
                               long long* request_id) {
    if (!s || !g || !force6n || !request_id || g->n_spheres <= 0 || !g->centers || !g->radii || !g->orders) {
        smob::set_last_error("null or empty request");
        return SMOB_ERR_ARG;
    }
    if (g->problem) {
        smob::set_last_error("a request is one problem: problem ids are not accepted");
        return SMOB_ERR_ARG;
    }
    if (!(tol > 0)) {
        smob::set_last_error("tolerance must be positive");
        return SMOB_ERR_ARG;
    }
    auto r = std::make_unique<Request>();
    const int n = g->n_spheres;
    r->n = n;
    r->centers.assign(g->centers, g->centers + 3 * n);
    r->radii.assign(g->radii, g->radii + n);
    r->orders.assign(g->orders, g->orders + n);
    if (g->quats) {
        r->has_quats = true;
        r->quats.assign(g->quats, g->quats + 4 * n);
    }
    r->force.assign(force6n, force6n + 6 * n);
    r->viscosity = g->viscosity;
    r->tol = tol;
    r->bytes = request_bytes(n, g->orders, s->opts.restart);
    std::lock_guard<std::mutex> lk(s->mu);
    if (double(r->bytes) > s->budget) {
        smob::set_last_error("request needs more device memory than the server budget");
        return SMOB_ERR_NOMEM;
    }
    r->id = s->next_id++;
    r->t_submit = s->now();
    *request_id = r->id;
    s->queue.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    s->cv.notify_all();
    return SMOB_OK;
}

static void fill_info(const Request* r, smob_request_info* info) {
    if (!info) return;
    info->state = r->state;
    info->status = r->status;
    info->t_submit = r->t_submit;
    info->t_admit = r->t_admit;
    info->t_done = r->t_done;
    info->bytes = double(r->bytes);
    info->stats = r->stats;
}

smob_status smob_server_poll(smob_server* s, long long id, double* vel6n, smob_request_info* info, int* done) {
    if (!s) return SMOB_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) {
        smob::set_last_error("unknown request id");
        return SMOB_ERR_ARG;
    }
    const Request* r = it->second.get();
    fill_info(r, info);
    if (done) *done = r->state == 2;
    if (r->state == 2 && vel6n && !r->vel.empty()) std::copy(r->vel.begin(), r->vel.end(), vel6n);
    if (r->state == 2 && r->status != SMOB_OK) smob::set_last_error(r->error.c_str());
    return SMOB_OK;
}

smob_status smob_server_wait(smob_server* s, long long id, double timeout_s, double* vel6n, smob_request_info* info) {
    if (!s) return SMOB_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) {
        smob::set_last_error("unknown request id");
        return SMOB_ERR_ARG;
    }
    // look the request up again on every wake-up: another thread may release it meanwhile
    const auto pred = [&] {
        auto f = s->reqs.find(id);
        return f == s->reqs.end() || f->second->state == 2;
    };
    if (timeout_s > 0) {
        if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
            smob::set_last_error("timed out waiting for the request");
            return SMOB_ERR_STATE;
        }
    } else {
        s->done_cv.wait(lk, pred);
    }
    it = s->reqs.find(id);
    if (it == s->reqs.end()) {
        smob::set_last_error("request was released while waiting for it");
        return SMOB_ERR_STATE;
    }
    const Request* r = it->second.get();
    fill_info(r, info);
    if (vel6n && !r->vel.empty()) std::copy(r->vel.begin(), r->vel.end(), vel6n);
    if (r->status != SMOB_OK) smob::set_last_error(r->error.c_str());
    return (smob_status)r->status;
}

smob_status smob_server_release(smob_server* s, long long id) {
    if (!s) return SMOB_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second->state != 2) {
        smob::set_last_error("request unknown or not finished");
        return SMOB_ERR_STATE;
    }
    s->reqs.erase(it);
    return SMOB_OK;
}

smob_status smob_server_stats(smob_server* s, smob_server_info* info) {
    if (!s || !info) return SMOB_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    info->queued = (int)s->queue.size();
    info->running = s->running;
    info->completed = s->completed;
    info->bytes_in_use = s->used;
    info->peak_bytes = s->peak_used;
    info->peak_running = s->peak_running;
    info->budget_bytes = s->budget;
    info->uptime_s = s->now();
    return SMOB_OK;
}

smob_status smob_server_destroy(smob_server* s) {
    if (!s) return SMOB_OK;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // let admitted requests finish; drop the queue
        s->queue.clear();
        s->done_cv.wait(lk, [&] { return s->running == 0; });
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
    return SMOB_OK;
}

}  // extern "C"
