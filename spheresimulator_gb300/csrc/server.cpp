// server.cpp — request loop for mobility solves with continuous batching on one GPU.
//
// The reference solves one system at a time inside SphereSystem::resolveCollision
// (SRC/SphereSystem.cpp:403-479); this server accepts independent mobility problems as they
// arrive and keeps several of them on the GPU at once:
//   * submit() copies the request (geometry, forces, tolerance) into one of two FIFO queues, small
//     requests (fewer than 1e9 far-field pairs) and big ones, and returns at once;
//   * worker threads (one per slot) admit a queue head when a slot is free and its device-memory
//     footprint fits in the budget left by the requests already on the GPU; the small queue goes
//     first, and big requests hold at most max_slots minus a reserve of a quarter of the slots (at
//     least one), so a small request never waits for a big one to finish;
//   * an admitted request gets its own context on its own non-blocking stream, so its kernels overlap
//     with the other requests' kernels on the device while its Krylov state stays device-resident;
//   * contexts allocate with the stream-ordered allocator, so admitting or retiring a request never
//     synchronizes the device;
//   * each request is solved exactly as it would be alone (its own context, deterministic kernels),
//     so results do not depend on what else is in flight;
//   * optionally (smob_server_partition) the device's SMs are split with green contexts: a small
//     partition that small requests use while a big request is running, and the rest for big
//     requests. A small request then never waits behind the long CTAs of a big one (FP64 near-field
//     and sphere kernels run for milliseconds per CTA), which stream priorities alone cannot prevent:
//     a running CTA is never preempted.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
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
smob_status create_context(smob_ctx** out, const smob_geometry* geo, int device, int priority_rank,
                           void* green_ctx);
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
    double t_submit = 0, t_admit = 0, t_ctx = 0, t_done = 0;
    smob_problem_stats stats{};
    std::string error;
    bool small = false;      // few far-field pairs (partition routing, stream priority)
    int route = 0;           // 0 whole device, 1 small partition, 2 big partition
};

// Green-context driver functions, reached through the runtime (the library does not link libcuda)
template <typename F>
F driver_fn(const char* name, unsigned version) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion(name, &f, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        f = nullptr;
    cudaGetLastError();
    return reinterpret_cast<F>(f);
}

// far-field pairs of a request below this: a small request
constexpr double kSmallPairs = 1e9;

// Streams share the device's hardware work queues (8 unless CUDA_DEVICE_MAX_CONNECTIONS says
// otherwise); kernels of streams mapped to one queue run in order, so with the server's many streams
// a small request's kernel would wait behind a big request's long kernel that happens to share its
// queue. The library asks for the maximum, 32, when it is loaded, unless the process has set the
// variable itself; it takes effect if no CUDA context exists yet in the process.
struct DeviceConnectionsDefault {
    DeviceConnectionsDefault() { setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0); }
};
DeviceConnectionsDefault g_device_connections_default;

}  // namespace

struct smob_server {
    smob_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv;       // workers wait for admissible work
    std::condition_variable done_cv;  // waiters wait for completions
    std::deque<long long> queue;      // small requests
    std::deque<long long> queue_big;  // big requests
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::vector<std::thread> workers;
    bool stop = false;
    long long next_id = 1;
    double budget = 0, used = 0, peak_used = 0;
    int running = 0, peak_running = 0;
    // SM partition (green contexts): small requests while a big one runs, and big requests
    CUgreenCtx g_small = nullptr, g_big = nullptr;
    int small_sms = 0, big_sms = 0;
    int running_big = 0;
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
                // big requests leave a quarter of the slots (at least one) to small ones
                const int big_cap = opts.max_slots > 1 ? opts.max_slots - std::max(1, opts.max_slots / 4) : 1;
                auto fits = [&](const std::deque<long long>& q) {
                    return !q.empty() && (used + double(reqs[q.front()]->bytes) <= budget || running == 0);
                };
                std::deque<long long>* from = nullptr;
                cv.wait(lk, [&] {
                    if (stop) return true;
                    if (fits(queue)) from = &queue;
                    else if (running_big < big_cap && fits(queue_big)) from = &queue_big;
                    else from = nullptr;
                    return from != nullptr;
                });
                if (stop) return;
                r = reqs[from->front()].get();
                from->pop_front();
                if (g_small) r->route = r->small ? (running_big > 0 ? 1 : 0) : 2;
                if (!r->small) ++running_big;
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
                if (!r->small) --running_big;
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
        const int rank = pairs < kSmallPairs ? 0 : (pairs < 3e10 ? 1 : 2);
        void* green = r->route == 1 ? static_cast<void*>(g_small) : (r->route == 2 ? static_cast<void*>(g_big) : nullptr);
        smob_status s = smob::create_context(&ctx, &g, opts.device, rank, green);
        r->t_ctx = now();
        // a request context solves once: capturing its graphs costs a small request more than replaying
        // them saves; a big one gains from the one-launch solve (graphs 2: big requests only)
        if (s == SMOB_OK && (opts.graphs == 0 || (opts.graphs == 2 && r->small))) s = smob_set_graphs(ctx, 0);
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
    b += size_t(128) * M;                     // their tensor-core strengths' split partials (4 x 16 B per
                                              // coarse point, up to ~2 coarse points per grid point)
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
    if (o->graphs < 0 || o->graphs > 2) {
        smob::set_last_error("server options: graphs must be 0 (none), 1 (all requests) or 2 (big requests)");
        return SMOB_ERR_ARG;
    }
    // Freed device memory stays in the device's stream-ordered pool instead of going back to the driver
    // at every synchronisation: requests allocate and free gigabytes while others run, and returning and
    // re-mapping that memory each time would stall the other requests' streams.
    // The pool may not hand a block freed on one request's stream to another request's allocation by
    // making the second stream wait for the first (the pool's "internal dependencies"): a small request
    // would then wait for whatever a big request had queued before its free, seconds of kernels.
    // Blocks whose free has completed on the device are still reused across streams.
    if (cudaSetDevice(o->device) == cudaSuccess) {
        cudaMemPool_t pool = nullptr;
        if (cudaDeviceGetDefaultMemPool(&pool, o->device) == cudaSuccess) {
            unsigned long long keep = ~0ULL;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            int no = 0;
            cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
        }
    }
    cudaGetLastError();
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
    double pts = 0;
    for (int i = 0; i < n; ++i) pts += double(g->orders[i] + 1) * (2 * g->orders[i] + 2);
    r->small = pts * pts < kSmallPairs;
    std::lock_guard<std::mutex> lk(s->mu);
    if (double(r->bytes) > s->budget) {
        smob::set_last_error("request needs more device memory than the server budget");
        return SMOB_ERR_NOMEM;
    }
    r->id = s->next_id++;
    r->t_submit = s->now();
    *request_id = r->id;
    (r->small ? s->queue : s->queue_big).push_back(r->id);
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
    info->t_ctx = r->t_ctx;
    info->route = r->route;
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
    info->queued = (int)(s->queue.size() + s->queue_big.size());
    info->running = s->running;
    info->completed = s->completed;
    info->bytes_in_use = s->used;
    info->peak_bytes = s->peak_used;
    info->peak_running = s->peak_running;
    info->budget_bytes = s->budget;
    info->uptime_s = s->now();
    return SMOB_OK;
}

static void drop_partition(smob_server* s) {
    using DestroyFn = CUresult (*)(CUgreenCtx);
    static DestroyFn destroy = driver_fn<DestroyFn>("cuGreenCtxDestroy", 12040);
    if (destroy) {
        if (s->g_small) destroy(s->g_small);
        if (s->g_big) destroy(s->g_big);
    }
    s->g_small = s->g_big = nullptr;
    s->small_sms = s->big_sms = 0;
}

smob_status smob_server_partition(smob_server* s, int small_sms) {
    if (!s || small_sms < 0) {
        smob::set_last_error("smob_server_partition: null server or negative SM count");
        return SMOB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running > 0 || !s->queue.empty() || !s->queue_big.empty()) {
        smob::set_last_error("smob_server_partition: the server must be idle (no queued or running requests)");
        return SMOB_ERR_STATE;
    }
    drop_partition(s);
    if (small_sms == 0) return SMOB_OK;
    using GetFn = CUresult (*)(CUdevice*, int);
    using ResFn = CUresult (*)(CUdevice, CUdevResource*, CUdevResourceType);
    using SplitFn = CUresult (*)(CUdevResource*, unsigned*, const CUdevResource*, CUdevResource*, unsigned, unsigned);
    using DescFn = CUresult (*)(CUdevResourceDesc*, CUdevResource*, unsigned);
    using CreateFn = CUresult (*)(CUgreenCtx*, CUdevResourceDesc, CUdevice, unsigned);
    const auto get = driver_fn<GetFn>("cuDeviceGet", 12000);
    const auto res = driver_fn<ResFn>("cuDeviceGetDevResource", 12040);
    const auto split = driver_fn<SplitFn>("cuDevSmResourceSplitByCount", 12040);
    const auto desc = driver_fn<DescFn>("cuDevResourceGenerateDesc", 12040);
    const auto create = driver_fn<CreateFn>("cuGreenCtxCreate", 12040);
    if (!get || !res || !split || !desc || !create) {
        smob::set_last_error("smob_server_partition: green contexts are not available from this driver");
        return SMOB_ERR_CUDA;
    }
    if (cudaSetDevice(s->opts.device) != cudaSuccess || cudaFree(nullptr) != cudaSuccess) {
        cudaGetLastError();
        smob::set_last_error("smob_server_partition: no usable device");
        return SMOB_ERR_NO_DEVICE;
    }
    CUdevice dev = 0;
    CUdevResource all{}, part{}, rest{};
    unsigned groups = 1;
    CUdevResourceDesc d_small{}, d_big{};
    if (get(&dev, s->opts.device) != CUDA_SUCCESS || res(dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS) {
        smob::set_last_error("smob_server_partition: cannot read the device's SM resource");
        return SMOB_ERR_CUDA;
    }
    if (unsigned(small_sms) + all.sm.minSmPartitionSize > all.sm.smCount) {
        smob::set_last_error("smob_server_partition: the small partition leaves too few SMs for the big one");
        return SMOB_ERR_ARG;
    }
    // the split rounds small_sms up to the partition granularity (8 SMs on GB300)
    if (split(&part, &groups, &all, &rest, 0, unsigned(small_sms)) != CUDA_SUCCESS || groups != 1 ||
        desc(&d_small, &part, 1) != CUDA_SUCCESS || desc(&d_big, &rest, 1) != CUDA_SUCCESS ||
        create(&s->g_small, d_small, dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS ||
        create(&s->g_big, d_big, dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS) {
        drop_partition(s);
        smob::set_last_error("smob_server_partition: splitting the SMs into green contexts failed");
        return SMOB_ERR_CUDA;
    }
    s->small_sms = int(part.sm.smCount);
    s->big_sms = int(rest.sm.smCount);
    return SMOB_OK;
}

smob_status smob_server_partition_info(smob_server* s, int* small_sms, int* big_sms) {
    if (!s) return SMOB_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (small_sms) *small_sms = s->small_sms;
    if (big_sms) *big_sms = s->big_sms;
    return SMOB_OK;
}

smob_status smob_server_destroy(smob_server* s) {
    if (!s) return SMOB_OK;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // let admitted requests finish; drop the queues
        s->queue.clear();
        s->queue_big.clear();
        s->done_cv.wait(lk, [&] { return s->running == 0; });
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    drop_partition(s);
    delete s;
    return SMOB_OK;
}

}  // extern "C"
