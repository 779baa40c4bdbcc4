// api.cu — host runtime of libsmob: context set-up, operator application, the batched
// restarted GMRES / iterative-refinement driver and the C ABI declared in include/smob.h.
//
// Reference counterparts:
//   SphereSTKSHOperator ctor / setupDOF / setupFMM / setupNearEval (BIE/SphereSTKSHOperator.cpp:7-144,539-573)
//     -> smob_create (grid, weights, normals, neighbour list, far-field work items, tables)
//   SphereSTKSHOperator::apply / applyP2POP / applyLOP / projectNullSpace (:153-521)
//     -> smob_apply / smob_apply_p2p / smob_apply_lop / smob_project_null_space
//   SphereSTKMobMat::solveMob / apply (BIE/SphereSTKMobMat.cpp:98-286) -> smob_solve_mob / smob_mob_apply
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/smob.h"
#include "krylov.h"
#include "sh_host.h"
#include "smob_internal.h"
#include "tc_sm100.h"

using namespace smob;

namespace smob {
smob_status create_context(smob_ctx** out, const smob_geometry* geo, int device, int priority_rank,
                           void* green_ctx = nullptr);
}

namespace {

thread_local std::string g_err;

struct SmobError : std::runtime_error {
    smob_status code;
    SmobError(smob_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CUDA_OK(expr)                                                                                   \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            throw SmobError(e_ == cudaErrorMemoryAllocation ? SMOB_ERR_NOMEM : SMOB_ERR_CUDA,          \
                            std::string(#expr) + ": " + cudaGetErrorString(e_));                        \
        }                                                                                               \
    } while (0)

// Stream that device buffers of the current call are allocated and freed on. Buffers use the
// stream-ordered allocator (cudaMallocAsync / cudaFreeAsync) so that creating or destroying one
// context never synchronizes the device: concurrent solves on other streams keep running.
thread_local cudaStream_t g_alloc_stream = nullptr;

struct AllocStreamScope {
    cudaStream_t prev;
    explicit AllocStreamScope(cudaStream_t s) : prev(g_alloc_stream) { g_alloc_stream = s; }
    ~AllocStreamScope() { g_alloc_stream = prev; }
};

// device buffer (RAII)
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = nullptr;  // stream the buffer was allocated on (freed on the same stream)
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t b) {
        if (b <= bytes && p) return;
        // an allocation inside a stream capture would become graph-owned memory that the buffer
        // then outlives: every buffer a captured pass uses is allocated before the capture
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (g_alloc_stream && cudaStreamIsCapturing(g_alloc_stream, &cs) == cudaSuccess &&
            cs != cudaStreamCaptureStatusNone)
            throw SmobError(SMOB_ERR_STATE, "device buffer allocation inside a graph capture");
        release();
        if (b == 0) b = 16;
        s = g_alloc_stream;
        CUDA_OK(cudaMallocAsync(&p, b, s));
        bytes = b;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
    template <typename T>
    void upload(const std::vector<T>& v) {
        alloc(v.size() * sizeof(T));
        if (!v.empty()) CUDA_OK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
};

// owns the context's stream; declared first in smob_ctx so it is destroyed after every buffer
struct StreamHolder {
    cudaStream_t st = nullptr;
    ~StreamHolder() {
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    }
};

// Pinned host staging for every copy between the host and a context's stream. A device-to-host copy
// into pageable memory blocks its thread until the stream reaches the copy, and the driver stages
// pageable copies through buffers the whole process shares: while one server request waits there
// for seconds of its own queued kernels, the other requests' pageable copies (a few bytes of solver
// state per Krylov block) wait with it. Pinned copies are plain stream-ordered DMA.
// Blocks come from a process-wide free list (portable, so any context, green ones included, may use
// them) and go back to it when the context is destroyed: freeing pinned memory can synchronize the
// device, which a server with requests in flight must not do.
std::mutex g_pin_mu;
std::multimap<size_t, void*> g_pin_free;

void* pin_acquire(size_t bytes, size_t* cap) {
    size_t want = 64 << 10;
    while (want < bytes) want <<= 1;
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        auto it = g_pin_free.lower_bound(want);
        if (it != g_pin_free.end()) {
            void* p = it->second;
            *cap = it->first;
            g_pin_free.erase(it);
            return p;
        }
    }
    void* p = nullptr;
    CUDA_OK(cudaHostAlloc(&p, want, cudaHostAllocPortable));
    *cap = want;
    return p;
}

void pin_release(void* p, size_t cap) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pin_free.emplace(cap, p);
}

// A context's staging block, handed out by bumping an offset; the offset goes back to 0 only after
// the context's stream was synchronized, so a host-to-device copy's source stays untouched until the
// copy ran without the host waiting for it.
struct HostStage {
    char* p = nullptr;
    size_t cap = 0, used = 0;
    HostStage() = default;
    HostStage(const HostStage&) = delete;
    HostStage& operator=(const HostStage&) = delete;
    ~HostStage() { pin_release(p, cap); }
};

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr int kGraphBlock = 4;  // Arnoldi steps per captured graph / per host check of the stop flags
// FP32 far field from coarse equivalent sources: per-pair tolerance (relative to the source sphere's
// contribution) and the coarse orders a sphere may use, ascending
// FP32 passes: they feed inner solves that stop at 1e-5 relative and FP32 residual updates of
// corrections below 1e-4 |b|, so their operator error only has to stay well below 1e-5. At 1e-5 the FP32
// far field's error against the FP64 sum is 2.8e-6 on cfg2 (1.0e-6 for the direct FP32 sum, 7.6e-7 at
// 1e-6), a residual update's error at most ~3e-10 |b|, and cfg2 solves take the same iterations,
// refinements and final error as at 1e-6 or 1e-4
constexpr double kCoarseEpsDefault = 1e-5;
// float-float passes (refinement residuals, u_hp): one decade below the 1e-8 solve tolerance. The mixed
// solves' velocity errors against the oracle's 1e-12 solves stay where the solve tolerance puts them
// from 1e-12 up to 9e-10 (cfg2 9.28e-11; 48 polydisperse spheres with near-singular gaps 6.68e-10; an
// uneven batch of 6 1.80e-10; 20 spheres at p = 24 4.05e-10, the same to three digits at 1e-10, 3e-10
// and 9e-10), while 1e-9 evaluates 22% fewer float-float pairs than 1e-10 on cfg2 (12.6 vs 13.8 ms
// per solve)
constexpr double kCoarseEpsHpDefault = 1e-9;
constexpr double kCoarseMargin = 1.0;  // orders added to log(eps) / log(a_s / r_min) (measured, p = 16)
// coarse targets: one order more (the traction's target normal raises the field's degree by one;
// with it the interpolated traction stays within the sources' error, measured in numpy over p = 12-24)
constexpr double kCoarseTargetMargin = 2.0;
constexpr int kCoarseLadder[] = {3, 4, 5, 6, 8, 10, 12, 14, 16, 20, 24, 28};
// recycled solutions (warm_start 2): pairs (force_i, mu_i) of earlier solves kept per context, with
// the forces orthonormalised per problem; a force closer than this (relative) to their span adds nothing
constexpr int kRecycleMax = 16;
constexpr double kRecycleDrop = 1e-10;
// parts of a recycled solve state: mu; and from MIXED solves the final residual r, the single layer
// u_hp at the last high-precision residual and that residual's mu (x_hp), all linear in the force
constexpr int kRecycleParts = 4;
// MIXED: a recycled guess whose residual is estimated below this (relative) is checked with the
// high-precision pass at once (it may already meet the tolerance), not with an FP32 residual
constexpr double kRecycleHpFirst = 1e-3;

}  // namespace

namespace smob {
// lets entry points outside this file report their message through smob_last_error()
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace smob

struct smob_ctx {
    StreamHolder sh;   // first member: destroyed last, after all buffers were freed on it
    StreamHolder sh2;  // side stream of the operator passes (far field beside sphere/near kernels)
    HostStage stage;   // pinned staging of the copies on st (smob_destroy synchronizes st first)
    int device = 0;
    cudaStream_t st = nullptr, st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int N = 0, M = 0, P = 0, pmax = 0;
    double viscosity = 1.0;
    std::vector<double> centers, radii, quats, weights;
    mutable std::vector<double> coords, norms;  // host copies, refreshed on demand after a geometry update
    std::vector<int> orders, prob, gidx, glen, coff, sid;
    std::vector<Problem> problems;
    std::vector<int> nbr_start, nbr_src, near_src_slot, slot_sphere;
    std::vector<unsigned char> nbr_precise;
    std::vector<double> org;         // per-problem origin of the relative (far-field) coordinates
    std::vector<char> map_orders;    // orders whose near maps are on the device
    mutable bool host_grid_stale = false;  // coords/norms changed on the device (geometry update)
    int n_precise = 0;
    int ncoef_total = 0;  // complex numbers
    long long set_stride_trac = 0, set_stride_sl = 0;
    std::vector<FarItem> items32, items64;
    std::vector<FarItem> items_tpt[3];  // FP32 item lists for 1, 2, 4 targets per thread
    std::vector<FarItem> items_df;      // float-float items: 2 * kFarThreadsDF targets
    int tpt = 2;                         // FP32 targets per thread chosen by the autotuner
    bool tuned = false;                  // autotuner run (or the tile set by the caller)
    double tune_ms[3] = {0, 0, 0};
    bool tune_cached = false;
    long long partial32 = 0, partial64 = 0;
    std::vector<VecChunk> chunks;
    // several right-hand sides: this context holds nrep copies of one problem (rep_M points each),
    // replica 0's FP32 far-field items drive the shared-geometry kernel
    int nrep = 1, rep_M = 0;
    std::vector<FarItem> items_rep;
    std::map<int, smob_ctx*> multi;  // replicated children of a one-problem context, by column count

    // device geometry
    DBuf d_center, d_radius, d_quat, d_order, d_gidx, d_glen, d_coff, d_prob, d_coords, d_norms, d_weights, d_sid;
    DBuf d_pos32, d_nrm32, d_pos32lo, d_nrm32lo, d_pos64, d_nrm64, d_nbr_start, d_nbr_src, d_nbr_precise, d_near_slot,
        d_slot_sphere, d_problems, d_tabs, d_srcdf, d_org;
    DBuf d_tab_d, d_tab_f, d_map_rowptr, d_map_col, d_map_val_d, d_map_val_f, d_items32, d_items64, d_items_df, d_chunks,
        d_items_rep;
    DBuf d_active;
    DBuf d_err;            // device error word (DevGeom::err)
    bool near_tc = true;   // FP32 near field on the tensor cores
    // FP32 coarse GEMMs on the tensor cores: strengths (k_coarse_src_tc, split-K over 4 CTAs per tile)
    // and coarse-target interpolation (k_ct_interp_tc); smob_set_coarse_tc modes
    bool coarse_tc = true;         // strengths
    bool coarse_interp_tc = true;  // interpolation
    // FP32 sphere operator with the Legendre stage on the tensor cores: off by default, measured slower
    // than the single-kernel SIMT operator (three launches per pass against one; cfg2 2.1 vs 1.1 ms per
    // solve, a 64-problem batch 0.54 vs 0.21 ms per pass)
    bool sph_tc = false;
    int n_leg_tiles = 0;
    DBuf d_leg_tiles, d_leg_sph, d_leg_tab, d_leg_off, d_fgbuf, d_lopbuf;
    // operator workspace
    DBuf d_src32, d_src64, d_partial32, d_partial64, d_coef32, d_coef64, d_sets32, d_sets64;
    // far field from coarse equivalent sources: the FP32 set and the float-float set (eps <= 0: off)
    struct CoarseHost {
        double eps = 0;
        bool hp = false;  // float-float set: FP64 maps, hi/lo points and strengths
        std::vector<int4> clev;
        std::vector<int2> cent;
        int ncoarse = 0;
        std::vector<int4> cdesc, cgrp, cdesc_tc;
        std::vector<int2> gent;
        DBuf d_clev, d_cent, d_cpos32, d_cpos32lo, d_csrc, d_cmap, d_cdesc, d_cgrp, d_gent, d_cdesc_tc, d_cmapA;
        DBuf d_cpart, d_ctile_count;  // tensor-core strengths: split partials and per-tile counters
        // coarse targets: listed entries with their candidate sources, work items, partial sums and
        // the interpolation side
        bool ctgt = false;
        std::vector<CtEnt> ctent;
        std::vector<int> ctsrc, ctused;
        std::vector<CtWork> ct_work;
        std::vector<CtITile> ctitile;
        std::vector<int> ctient;
        // tensor-core interpolation (FP32 set): tiles of 128 grid points x up to kCoarseTcSph entries of
        // one map, their entry lists, and the maps' A operand pre-split and tiled (offset in the tile)
        std::vector<CtITile> ctitile_tc;
        std::vector<int> ctient_tc;
        DBuf d_ctitile_tc, d_ctient_tc, d_cmapI;
        long long ct_partial = 0;
        DBuf d_ctent, d_ctsrc, d_ctcand, d_ctused, d_ct_work, d_ct_partial, d_ctinterp, d_cmapT, d_cnrm32,
            d_cnrm32lo, d_ctu, d_ctitile, d_ctient;
    };
    CoarseHost c32, chp;
    DBuf d_cnode, d_cnode_off, d_sph32;
    smob_ctx() {
        c32.eps = kCoarseEpsDefault;
        c32.ctgt = true;
        chp.eps = kCoarseEpsHpDefault;
        chp.hp = true;
        chp.ctgt = true;
    }
    DBuf d_in, d_out, d_tmp;  // host-pointer API staging
    // solver workspace
    int restart_cap = 0;
    DBuf d_V, d_w, d_r, d_x, d_xlast, d_b, d_rho, d_u, d_force, d_vel;
    // mixed solve: rho + x, and the single layer of rho + x_hp at the last high-precision residual x_hp
    DBuf d_dens, d_uhp, d_xhp, d_partial64_sl;
    DBuf d_pz;  // preconditioned vector P v
    // recycled solutions: rq (host, orthonormal forces per problem, [kRecycleMax][6N]) and d_ru
    // (device, [kRecycleMax][kRecycleParts][3M]) the solve states transformed alike; rk columns of
    // each, all from solves of precision rprec
    std::vector<double> rq;
    DBuf d_ru, d_rcoef, d_rscale;
    int rk = 0, rprec = -1;
    DBuf d_H, d_g, d_cs, d_sn, d_y, d_kc, d_ks, d_norm, d_hn, d_beta, d_partial_red, d_incycle;
    // graph-driven restart loop: per-problem state, scalars and body counters, residual masks, the
    // Arnoldi step counter and per-step run counts
    DBuf d_track, d_sparams, d_updmask, d_hpmask, d_freshmask, d_jdev, d_runs_j, d_bnorm;
    DBuf d_red_count;     // per (problem, vector) counters of the fused dot reductions
    int red_cstride = 0;  // counters per problem
    bool have_xlast = false;

    DevGeom g{};
    long long launches = 0;    // kernels run (graph nodes included)
    long long host_calls = 0;  // launches issued from the host: kernels outside graphs and graph launches
    bool capturing = false;    // a stream capture of the context's work is open
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    DBuf d_flush;
    unsigned flush_val = 1;
    // captured Arnoldi blocks (see solve_device)
    struct Graph {
        cudaGraphExec_t exec;
        long long kernels;
    };
    bool use_graphs = true;
    std::map<long long, Graph> graphs;
    // the whole restart-cycle loop as one graph with device-side decisions (solve_device), per
    // (precisions, preconditioner, restart, iteration limit); kernels per body for the launch count
    struct LoopGraph {
        cudaGraphExec_t exec = nullptr;
        long long k_top = 0, k_cycle = 0, k_upd = 0, k_hp = 0;
        std::vector<long long> k_step;  // per step index j: step(j) and the step-control kernel
        long long k_post = 0, k_from = 0, k_moved = 0, k_fresh = 0;  // full-solve graph: final velocity
    };
    std::map<std::vector<int>, LoopGraph> loop_graphs;
    bool loop_graph_ok = true;  // false once building one failed (the host-driven loop runs instead)
    bool eps_hp_auto = true;    // the float-float set's tolerance follows the solves (fit_eps_hp)
    bool multi_shared = false;  // several right-hand sides: shared-pair kernels instead of a batch
    bool loop_graph_on = true;  // smob_set_loop_graph
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
        for (auto& kv : loop_graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        loop_graphs.clear();
    }

    // profiling
    bool prof = false;
    struct ProfRec {
        long long launches = 0;
        double ms = 0;
    };
    std::map<std::string, ProfRec> prof_tab;
    struct Pending {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;

    KrylovLaunch kl() {
        KrylovLaunch L;
        L.chunks = d_chunks.as<VecChunk>();
        L.nchunks = (int)chunks.size();
        L.problems = d_problems.as<Problem>();
        L.P = P;
        L.partial = d_partial_red.as<double>();
        L.partial_cap = (long long)(d_partial_red.bytes / sizeof(double));
        L.counters = d_red_count.as<unsigned>();
        L.cstride = red_cstride;
        return L;
    }

    ~smob_ctx() {
        for (auto& kv : multi) smob_destroy(kv.second);
        for (auto& p : pending) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        if (ev_a) cudaEventDestroy(ev_a);
        if (ev_b) cudaEventDestroy(ev_b);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        drop_graphs();
    }
};

namespace {

// ---------------------------------------------------------------- profiling helpers
struct ProfScope {
    smob_ctx* c;
    const char* name;
    cudaStream_t s;
    cudaEvent_t a{}, b{};
    ProfScope(smob_ctx* ctx, const char* n, cudaStream_t st = nullptr) : c(ctx), name(n), s(st ? st : ctx->st) {
        if (c->prof) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, s);
        }
    }
    ~ProfScope() {
        if (c->prof) {
            cudaEventRecord(b, s);
            c->pending.push_back({name, a, b});
        }
    }
};

// Fork/join of one operator pass: the far field runs on the side stream while the sphere and near
// kernels run on the main stream (they touch disjoint buffers until the far-field reduction, which
// follows the join). Serial when profiling, so each kernel's CUDA-event time stays its own.
struct PassFork {
    smob_ctx* c;
    bool on;
    explicit PassFork(smob_ctx* ctx) : c(ctx), on(ctx->st2 != nullptr && !ctx->prof) {
        if (on) {
            CUDA_OK(cudaEventRecord(c->ev_fork, c->st));
            CUDA_OK(cudaStreamWaitEvent(c->st2, c->ev_fork, 0));
        }
    }
    cudaStream_t far() const { return on ? c->st2 : c->st; }
    void join() {
        if (on) {
            CUDA_OK(cudaEventRecord(c->ev_join, c->st2));
            CUDA_OK(cudaStreamWaitEvent(c->st, c->ev_join, 0));
            on = false;
        }
    }
};

void prof_flush(smob_ctx* c) {
    if (c->pending.empty()) return;
    cudaStreamSynchronize(c->st);
    for (auto& p : c->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        auto& r = c->prof_tab[p.name];
        r.launches += 1;
        r.ms += ms;
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    c->pending.clear();
}

void check_launch(smob_ctx* c, int n) {
    if (n < 0) throw SmobError(SMOB_ERR_STATE, "kernel launch refused: more vectors than the work buffers hold");
    c->launches += n;
    if (!c->capturing) c->host_calls += n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw SmobError(SMOB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
}

// staging space of `bytes` in the context's pinned block, valid until the next stage_sync
void* stage_alloc(smob_ctx* c, size_t bytes) {
    bytes = (bytes + 15) & ~size_t(15);
    HostStage& h = c->stage;
    if (h.used + bytes > h.cap) {
        if (h.used > 0) {  // copies issued since the last synchronization may still use the block
            CUDA_OK(cudaStreamSynchronize(c->st));
            h.used = 0;
        }
        if (bytes > h.cap) {
            pin_release(h.p, h.cap);
            h.p = nullptr;
            h.cap = 0;
            size_t cap = 0;
            h.p = static_cast<char*>(pin_acquire(bytes, &cap));
            h.cap = cap;
        }
    }
    void* r = h.p + h.used;
    h.used += bytes;
    return r;
}

// the copies issued through the stage have run (their host destinations may be read)
void stage_sync(smob_ctx* c) {
    CUDA_OK(cudaStreamSynchronize(c->st));
    c->stage.used = 0;
}

// host to device on the context's stream without waiting: the source is copied into the stage first
void h2d(smob_ctx* c, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    void* s = stage_alloc(c, bytes);
    std::memcpy(s, src, bytes);
    CUDA_OK(cudaMemcpyAsync(dst, s, bytes, cudaMemcpyHostToDevice, c->st));
}

// device to host on the context's stream; returns when the data is in dst
void d2h(smob_ctx* c, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    void* s = stage_alloc(c, bytes);
    CUDA_OK(cudaMemcpyAsync(s, src, bytes, cudaMemcpyDeviceToHost, c->st));
    stage_sync(c);
    std::memcpy(dst, s, bytes);
}

// counters of the fused dot reductions: nvec per problem, zeroed (the kernels leave them zero)
void alloc_red_counters(smob_ctx* c, int nvec) {
    c->d_red_count.alloc(sizeof(unsigned) * (size_t)std::max(c->P, 1) * nvec);
    CUDA_OK(cudaMemsetAsync(c->d_red_count.p, 0, sizeof(unsigned) * (size_t)std::max(c->P, 1) * nvec, c->st));
    c->red_cstride = nvec;
}

// unit quaternion of sphere i from a caller's orientation: normalised, except that one already of
// unit norm (to 1e-15) is kept bit for bit, so a geometry read back and passed in again is reproduced
void unit_quat(const double* q, double* out, int i) {
    const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    const double nq = std::sqrt(n2);
    if (!(nq > 0) || !std::isfinite(nq))
        throw SmobError(SMOB_ERR_ARG, "quaternion of sphere " + std::to_string(i) + " is zero or not finite");
    for (int k = 0; k < 4; ++k) out[k] = std::fabs(n2 - 1.0) <= 1e-15 ? q[k] : q[k] / nq;
}

// ---------------------------------------------------------------- context set-up
// Spheres of one problem must not overlap or touch: checked on the device (k_overlap) for the
// centres d_centers with the context's radii and problems (d_radius, d_prob, d_problems uploaded);
// throws with the first such pair in (t, s) order and changes nothing.
void check_overlap(smob_ctx* c, const double* d_centers) {
    DBuf first;
    first.alloc(sizeof(unsigned long long));
    CUDA_OK(cudaMemsetAsync(first.p, 0xff, sizeof(unsigned long long), c->st));
    check_launch(c, launch_overlap_check(d_centers, c->d_radius.as<double>(), c->d_prob.as<int>(),
                                         c->d_problems.as<Problem>(), c->N, first.as<unsigned long long>(), c->st));
    unsigned long long h = 0;
    d2h(c, &h, first.p, sizeof(h));
    if (h != ~0ULL) {
        const long long t = (long long)(h / (unsigned long long)c->N), sp = (long long)(h % (unsigned long long)c->N);
        throw SmobError(SMOB_ERR_ARG, "spheres " + std::to_string(t) + " and " + std::to_string(sp) +
                                          " overlap or touch");
    }
}

// Near pairs (MPI/NearInteraction.txx:430-447; Rad = 1.5*radius, SphereSTKSHOperator.cpp:547) within
// each problem, built on the device from d_center (nbrlist.cu): CSR by target with sources ascending,
// near-singular flags, near-source slots in sphere order. The host keeps a copy of these O(N + pairs)
// arrays for the bookkeeping that reads them (near maps per order, coarse-level candidates, counts).
void build_near(smob_ctx* c) {
    const int N = c->N;
    DBuf count, totals;
    count.alloc(sizeof(int) * std::max(N, 1));
    totals.alloc(2 * sizeof(int));
    c->d_nbr_start.alloc(sizeof(int) * (N + 1));
    c->d_near_slot.alloc(sizeof(int) * std::max(N, 1));
    const double* ctr = c->d_center.as<double>();
    const double* rad = c->d_radius.as<double>();
    check_launch(c, launch_nbr_count(ctr, rad, c->d_prob.as<int>(), c->d_problems.as<Problem>(), N, count.as<int>(),
                                     c->st));
    check_launch(c, launch_nbr_scan(count.as<int>(), N, c->d_nbr_start.as<int>(), c->d_near_slot.as<int>(),
                                    totals.as<int>(), c->st));
    int tot[2] = {0, 0};
    d2h(c, tot, totals.p, sizeof(tot));
    c->d_nbr_src.alloc(sizeof(int) * std::max(tot[0], 1));
    c->d_nbr_precise.alloc(std::max(tot[0], 1));
    c->d_slot_sphere.alloc(sizeof(int) * std::max(tot[1], 1));
    check_launch(c, launch_nbr_fill(ctr, rad, c->d_prob.as<int>(), c->d_problems.as<Problem>(), N,
                                    c->d_nbr_start.as<int>(), c->d_near_slot.as<int>(), c->d_nbr_src.as<int>(),
                                    c->d_nbr_precise.as<unsigned char>(), c->d_slot_sphere.as<int>(), c->st));
    c->nbr_start.resize(N + 1);
    c->nbr_src.resize(tot[0]);
    c->nbr_precise.resize(tot[0]);
    c->near_src_slot.resize(N);
    c->slot_sphere.resize(tot[1]);
    // the lists in one staged batch: the copies, one synchronization, then the host mirrors
    struct Part {
        void* dst;
        const void* src;
        size_t bytes;
        void* staged;
    } parts[] = {{c->nbr_start.data(), c->d_nbr_start.p, sizeof(int) * (N + 1), nullptr},
                 {c->nbr_src.data(), c->d_nbr_src.p, sizeof(int) * tot[0], nullptr},
                 {c->nbr_precise.data(), c->d_nbr_precise.p, size_t(tot[0]), nullptr},
                 {c->near_src_slot.data(), c->d_near_slot.p, sizeof(int) * N, nullptr},
                 {c->slot_sphere.data(), c->d_slot_sphere.p, sizeof(int) * tot[1], nullptr}};
    size_t all = 0;
    for (const Part& q : parts) all += (q.bytes + 15) & ~size_t(15);
    stage_alloc(c, all);  // room for the whole batch (synchronizes or grows the block first if needed)
    c->stage.used -= all;
    for (Part& q : parts) {
        if (q.bytes == 0) continue;
        q.staged = stage_alloc(c, q.bytes);
        CUDA_OK(cudaMemcpyAsync(q.staged, q.src, q.bytes, cudaMemcpyDeviceToHost, c->st));
    }
    stage_sync(c);
    for (const Part& q : parts)
        if (q.bytes) std::memcpy(q.dst, q.staged, q.bytes);
}

void problem_origins(smob_ctx* c);
void upload_near(smob_ctx* c);
void build_tables(smob_ctx* c);
void build_leg(smob_ctx* c);
void bind_geom(smob_ctx* c);
void build_coarse(smob_ctx* c);
void coarse_grids(smob_ctx* c);

// source-sphere chunks of a problem's far-field work items: consecutive spheres of about
// max(2048, M_problem / 16) grid points; depends only on the problem itself, so its sums are the
// same alone or inside any batch
std::vector<std::pair<int, int>> source_chunks(const smob_ctx* c, const Problem& pr) {
    const int mp = pr.p1 - pr.p0;
    const int ch = std::max(2048, (mp + 15) / 16);
    std::vector<std::pair<int, int>> chunks;
    int cs = pr.s0, acc = 0;
    for (int s = pr.s0; s < pr.s1; ++s) {
        acc += c->glen[s];
        if (acc >= ch || s + 1 == pr.s1) {
            chunks.push_back({cs, s + 1});
            cs = s + 1;
            acc = 0;
        }
    }
    return chunks;
}

void build_context(smob_ctx* c, const smob_geometry* geo) {
    const int N = geo->n_spheres;
    c->N = N;
    c->viscosity = geo->viscosity;
    c->centers.assign(geo->centers, geo->centers + 3 * N);
    c->radii.assign(geo->radii, geo->radii + N);
    c->orders.assign(geo->orders, geo->orders + N);
    c->quats.resize(4 * N);
    for (int i = 0; i < N; ++i) {
        if (geo->quats) {
            unit_quat(geo->quats + 4 * i, &c->quats[4 * i], i);
        } else {
            c->quats[4 * i] = 1;
            c->quats[4 * i + 1] = c->quats[4 * i + 2] = c->quats[4 * i + 3] = 0;
        }
    }
    c->prob.resize(N);
    for (int i = 0; i < N; ++i) c->prob[i] = geo->problem ? geo->problem[i] : 0;
    for (int i = 0; i < N; ++i) {
        if (!(c->radii[i] > 0) || !std::isfinite(c->radii[i]))
            throw SmobError(SMOB_ERR_ARG, "radius of sphere " + std::to_string(i) + " must be positive and finite");
        if (c->orders[i] < 1 || c->orders[i] > kMaxOrder)
            throw SmobError(SMOB_ERR_ARG, "order of sphere " + std::to_string(i) + " outside [1, 32]");
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(c->centers[3 * i + k]))
                throw SmobError(SMOB_ERR_ARG, "centre of sphere " + std::to_string(i) + " is not finite");
        if (i > 0 && c->prob[i] < c->prob[i - 1]) throw SmobError(SMOB_ERR_ARG, "problem ids must be non-decreasing");
        if (c->prob[i] < 0) throw SmobError(SMOB_ERR_ARG, "problem ids must be >= 0");
    }
    if (N > 0 && c->prob[0] != 0) throw SmobError(SMOB_ERR_ARG, "problem ids must start at 0");
    for (int i = 1; i < N; ++i)
        if (c->prob[i] > c->prob[i - 1] + 1) throw SmobError(SMOB_ERR_ARG, "problem ids must be contiguous");
    c->P = N > 0 ? c->prob[N - 1] + 1 : 0;
    c->pmax = *std::max_element(c->orders.begin(), c->orders.end());

    // points and coefficient offsets
    c->gidx.resize(N);
    c->glen.resize(N);
    c->coff.resize(N);
    int off = 0, coffs = 0;
    for (int i = 0; i < N; ++i) {
        const int p = c->orders[i];
        c->gidx[i] = off;
        c->glen[i] = (p + 1) * (2 * p + 2);
        off += c->glen[i];
        c->coff[i] = coffs;
        coffs += 3 * ncoef(p);
    }
    c->M = off;
    c->ncoef_total = coffs;
    // grid points and normals are built on the device (launch_regrid, below) from the centres and
    // orientations, at creation and after every geometry update alike; the host copies follow on demand
    c->coords.resize(3 * off);
    c->norms.resize(3 * off);
    c->host_grid_stale = true;
    c->weights.resize(off);
    c->sid.resize(off);
    for (int i = 0; i < N; ++i) {
        const HostOrderTables& T = host_tables(c->orders[i]);
        const double a = c->radii[i];
        for (int j = 0; j < T.nt; ++j)
            for (int k = 0; k < T.nphi; ++k) {
                const int id = c->gidx[i] + j * T.nphi + k;
                c->weights[id] = a * a * T.wq[j];
                c->sid[id] = i;
            }
    }

    // problems
    c->problems.assign(c->P, Problem{});
    for (int p = 0; p < c->P; ++p) {
        c->problems[p].s0 = N;
        c->problems[p].s1 = 0;
    }
    for (int i = 0; i < N; ++i) {
        Problem& pr = c->problems[c->prob[i]];
        pr.s0 = std::min(pr.s0, i);
        pr.s1 = std::max(pr.s1, i + 1);
    }
    for (auto& pr : c->problems) {
        pr.p0 = c->gidx[pr.s0];
        pr.p1 = c->gidx[pr.s1 - 1] + c->glen[pr.s1 - 1];
        pr.v0 = 3 * pr.p0;
        pr.v1 = 3 * pr.p1;
    }

    // what the device neighbour list and overlap check read (the problems are uploaded again below,
    // with their far-field and reduction fields)
    c->d_center.upload(c->centers);
    c->d_radius.upload(c->radii);
    c->d_prob.upload(c->prob);
    c->d_problems.upload(c->problems);
    check_overlap(c, c->d_center.as<double>());
    build_near(c);
    const int ndmax = ncoef(c->pmax + 3);
    c->set_stride_trac = 2LL * kNearSetsTrac * ndmax;
    c->set_stride_sl = 2LL * kNearSetsSL * ndmax;

    // far-field work items: target blocks x source-sphere chunks; the chunking depends only on
    // the problem itself, so a problem's sums are identical alone or inside any batch
    auto make_items = [&](int tblock, std::vector<FarItem>& items, long long& partial_elems) {
        items.clear();
        long long poff = 0;
        for (int pi = 0; pi < c->P; ++pi) {
            Problem& pr = c->problems[pi];
            const int mp = pr.p1 - pr.p0;
            const std::vector<std::pair<int, int>> chunks = source_chunks(c, pr);
            pr.nchunks = (int)chunks.size();
            pr.poff = poff;
            poff += 3LL * mp * pr.nchunks;
            for (int t0 = pr.p0; t0 < pr.p1; t0 += tblock)
                for (int ci = 0; ci < pr.nchunks; ++ci)
                    items.push_back(FarItem{t0, std::min(t0 + tblock, pr.p1), chunks[ci].first, chunks[ci].second, pi, ci});
        }
        partial_elems = poff;
    };
    // both item lists share the chunking rule, so Problem.nchunks/poff are the same for both
    make_items(kFarTargets64, c->items64, c->partial64);
    for (int k = 0; k < 3; ++k) make_items(kFarThreads << k, c->items_tpt[k], c->partial32);
    {
        long long unused = 0;
        make_items(2 * kFarThreadsDF, c->items_df, unused);
    }
    c->items32 = c->items_tpt[1];
    // heavier problems first helps the tail of uneven batches
    auto by_cost = [&](std::vector<FarItem>& items) {
        std::stable_sort(items.begin(), items.end(), [&](const FarItem& a, const FarItem& b) {
            const Problem& pa = c->problems[a.problem];
            const Problem& pb = c->problems[b.problem];
            return (pa.p1 - pa.p0) > (pb.p1 - pb.p0);
        });
    };
    by_cost(c->items32);
    by_cost(c->items64);
    by_cost(c->items_df);
    for (auto& v : c->items_tpt) by_cost(v);

    // reduction chunks for the Krylov vectors
    c->chunks.clear();
    for (int pi = 0; pi < c->P; ++pi) {
        Problem& pr = c->problems[pi];
        pr.c0 = (int)c->chunks.size();
        for (long long l = pr.v0; l < pr.v1; l += kVecChunk)
            c->chunks.push_back(VecChunk{l, std::min<long long>(l + kVecChunk, pr.v1), pi, 0});
        pr.c1 = (int)c->chunks.size();
    }

    build_tables(c);
    build_leg(c);

    // point data: FP64 lab-frame grid and the far-field copies relative to each problem's origin
    // (centre of its sphere bounding box), all written by the regrid kernel below
    problem_origins(c);
    c->d_center.upload(c->centers);
    c->d_radius.upload(c->radii);
    c->d_quat.upload(c->quats);
    c->d_order.upload(c->orders);
    c->d_gidx.upload(c->gidx);
    c->d_glen.upload(c->glen);
    c->d_coff.upload(c->coff);
    c->d_prob.upload(c->prob);
    c->d_coords.alloc(sizeof(double) * 3 * c->M);
    c->d_norms.alloc(sizeof(double) * 3 * c->M);
    c->d_weights.upload(c->weights);
    c->d_sid.upload(c->sid);
    c->d_pos32.alloc(sizeof(float4) * c->M);
    c->d_nrm32.alloc(sizeof(float4) * c->M);
    c->d_pos32lo.alloc(sizeof(float4) * c->M);
    c->d_nrm32lo.alloc(sizeof(float4) * c->M);
    c->d_pos64.alloc(sizeof(double4_32a) * c->M);
    c->d_nrm64.alloc(sizeof(double4_32a) * c->M);
    c->d_org.upload(c->org);
    c->d_problems.upload(c->problems);
    c->d_items32.upload(c->items32);
    c->d_items64.upload(c->items64);
    c->d_items_df.upload(c->items_df);  // float-float far field: 2 targets per thread
    c->d_chunks.upload(c->chunks);
    std::vector<unsigned char> act(c->P, 1);
    c->d_active.upload(act);
    c->d_err.alloc(sizeof(int));
    CUDA_OK(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->st));

    // operator workspace
    c->d_src32.alloc(sizeof(float4) * c->M);
    c->d_src64.alloc(sizeof(double4_32a) * c->M);
    c->d_srcdf.alloc(sizeof(float4) * 2 * c->M);
    c->d_partial32.alloc(sizeof(float) * c->partial32);
    c->d_partial64.alloc(sizeof(double) * c->partial64);
    c->d_coef32.alloc(sizeof(float) * 2 * c->ncoef_total);
    c->d_coef64.alloc(sizeof(double) * 2 * c->ncoef_total);
    c->d_in.alloc(sizeof(double) * 3 * c->M);
    c->d_out.alloc(sizeof(double) * 3 * c->M);
    c->d_tmp.alloc(sizeof(double) * 3 * c->M);
    c->d_partial_red.alloc(sizeof(double) * c->chunks.size() * 2);
    alloc_red_counters(c, 2);
    upload_near(c);
    build_coarse(c);
    bind_geom(c);
    check_launch(c, launch_regrid(c->g, c->d_org.as<double>(), c->st));
    coarse_grids(c);
}

// ---------------------------------------------------------------- tables, near metadata, bindings
// per-problem origin for the relative point coordinates: centre of the problem's sphere bounding box
void problem_origins(smob_ctx* c) {
    c->org.assign(3 * c->P, 0.0);
    for (int pi = 0; pi < c->P; ++pi) {
        const Problem& pr = c->problems[pi];
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int s = pr.s0; s < pr.s1; ++s)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], c->centers[3 * s + k]);
                hi[k] = std::max(hi[k], c->centers[3 * s + k]);
            }
        for (int k = 0; k < 3; ++k) c->org[3 * pi + k] = 0.5 * (lo[k] + hi[k]);
    }
}

// the near-set workspace for this geometry's near sources; near lanes of the SIMT near kernel
void upload_near(smob_ctx* c) {
    // (the lists themselves were built on the device by build_near)
    c->n_precise = 0;
    for (unsigned char v : c->nbr_precise) c->n_precise += v;
    const size_t nsl = c->slot_sphere.size();
    // FP32 sets: [idx][set] for the SIMT kernel or the tiles of the tensor-core kernel, whose padding
    // must read as zero (cleared here, on every geometry update and when the near kernel is switched)
    const long long s32 = std::max({c->set_stride_trac, c->set_stride_sl, near_tile_stride(c->pmax, true),
                                    near_tile_stride(c->pmax, false)});
    c->d_sets32.alloc(sizeof(float) * std::max<size_t>(nsl, 1) * s32);
    CUDA_OK(cudaMemsetAsync(c->d_sets32.p, 0, c->d_sets32.bytes, c->st));
    c->d_sets64.alloc(sizeof(double) * nsl * std::max(c->set_stride_trac, c->set_stride_sl));
    // near-field lanes per target: ~152 x 256 threads when few target points have near pairs (the
    // kernel runs beside the far field, which fills the rest of the GPU; more lanes repeat the
    // recurrence: with the sets in shared memory, cfg2 solves take 20.5 ms with 2 lanes, 21.0 with 4,
    // 21.4 with 8 and 22.1 with 1), one lane (no repeated recurrence) when many do; the lane count does
    // not change any result (each set is summed by one lane in a fixed order)
    long long tpts = 0;
    for (int t = 0; t < c->N; ++t)
        if (c->nbr_start[t + 1] > c->nbr_start[t]) tpts += c->glen[t];
    const double want = 152.0 * 256.0 / double(std::max<long long>(tpts, 1));
    c->g.near_lanes = want >= 8 ? 8 : (want >= 4 ? 4 : (want >= 2 ? 2 : 1));
}

// transform tables of every order present, near maps of the orders of near-source spheres
void build_tables(smob_ctx* c) {
    std::vector<OrderTables> tabs(kMaxOrder + 1);
    std::vector<double> tab;
    std::vector<int> rowptr, col;
    std::vector<double> mval;
    std::vector<char> present(kMaxOrder + 1, 0);
    for (int p : c->orders) present[p] = 1;
    for (int p = 1; p <= kMaxOrder; ++p) {
        if (!present[p]) continue;
        const HostOrderTables& T = host_tables(p);
        OrderTables& o = tabs[p];
        o.p = p;
        o.nt = T.nt;
        o.nphi = T.nphi;
        o.nc = T.nc;
        o.ring = (int)tab.size();
        tab.insert(tab.end(), T.ct.begin(), T.ct.end());
        tab.insert(tab.end(), T.st.begin(), T.st.end());
        tab.insert(tab.end(), T.wq.begin(), T.wq.end());
        o.leg = (int)tab.size();
        tab.insert(tab.end(), T.P.begin(), T.P.end());
        tab.insert(tab.end(), T.dP.begin(), T.dP.end());
        tab.insert(tab.end(), T.Ps.begin(), T.Ps.end());
        o.twiddle = (int)tab.size();
        tab.insert(tab.end(), T.cosmk.begin(), T.cosmk.end());
        tab.insert(tab.end(), T.sinmk.begin(), T.sinmk.end());
        o.cph = (int)tab.size();
        tab.insert(tab.end(), T.cph.begin(), T.cph.end());
        tab.insert(tab.end(), T.sph.begin(), T.sph.end());
        o.trac_map = o.sl_map = -1;
        o.trac_rows = o.sl_rows = 0;
    }
    // near maps only for orders of spheres that are near sources
    std::vector<char> near_p(kMaxOrder + 1, 0);
    for (int s : c->slot_sphere) near_p[c->orders[s]] = 1;
    rowptr.clear();
    for (int p = 1; p <= kMaxOrder; ++p) {
        if (!near_p[p]) continue;
        for (int kind = 0; kind < 2; ++kind) {
            const SparseMap& mp = near_map(p, kind == 0);
            const int base = (int)rowptr.size();
            const int e0 = (int)col.size();
            for (int r = 0; r < mp.rows; ++r) rowptr.push_back(e0 + mp.rowptr[r]);
            rowptr.push_back(e0 + mp.rowptr[mp.rows]);
            col.insert(col.end(), mp.col.begin(), mp.col.end());
            mval.insert(mval.end(), mp.val.begin(), mp.val.end());
            if (kind == 0) {
                tabs[p].trac_map = base;
                tabs[p].trac_rows = mp.rows;
            } else {
                tabs[p].sl_map = base;
                tabs[p].sl_rows = mp.rows;
            }
        }
    }
    std::vector<double> c1, c2, dg;
    theta_recurrence(kMaxOrder + 4, c1, c2, dg);
    c->g.th_c1 = (int)tab.size();
    tab.insert(tab.end(), c1.begin(), c1.end());
    c->g.th_c2 = (int)tab.size();
    tab.insert(tab.end(), c2.begin(), c2.end());
    c->g.th_diag = (int)tab.size();
    tab.insert(tab.end(), dg.begin(), dg.end());

    c->d_tabs.upload(tabs);
    c->d_tab_d.upload(tab);
    std::vector<float> tabf(tab.begin(), tab.end());
    c->d_tab_f.upload(tabf);
    c->d_map_rowptr.upload(rowptr);
    c->d_map_col.upload(col);
    c->d_map_val_d.upload(mval);
    std::vector<float> mvalf(mval.begin(), mval.end());
    c->d_map_val_f.upload(mvalf);
    c->map_orders = near_p;
}

// Tensor-core Legendre stage of the FP32 sphere operator (k_legendre_tc): tiles of up to 21 spheres of
// one order, and per present order p and m the B operand tables in the tc_sm100.h operand layout,
// chunks of 32 K values: forward rows n = m..p (padded to 16), K = (block b, ring j) -> w_j times P, dP
// or m Ps at (j, n, m); inverse rows j = 0..p (padded to 16), K = (block b, n - m) -> the same tables
// unweighted. Depends only on the orders.
void build_leg(smob_ctx* c) {
    constexpr int kSpt = 21, kK = 32;
    std::vector<int4> tiles;
    std::vector<int> sph;
    std::vector<float> tab;
    std::vector<int> off(2 * (kMaxOrder + 1) * (kMaxOrder + 1), 0);
    auto kmaj = [](int r, int k) { return ((r >> 3) * (kK >> 2) + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3); };
    for (int p = 1; p <= kMaxOrder; ++p) {
        std::vector<int> list;
        for (int i = 0; i < c->N; ++i)
            if (c->orders[i] == p) list.push_back(i);
        if (list.empty()) continue;
        for (size_t a = 0; a < list.size(); a += kSpt)
            tiles.push_back(make_int4(p, (int)(sph.size() + a), (int)std::min<size_t>(kSpt, list.size() - a), 0));
        sph.insert(sph.end(), list.begin(), list.end());
        const HostOrderTables& T = host_tables(p);
        const int nt = p + 1, nc = T.nc;
        const int KP = kK * ((3 * nt + kK - 1) / kK), nch = KP / kK;
        for (int m = 0; m <= p; ++m) {
            const int nn = p + 1 - m;
            for (int dir = 0; dir < 2; ++dir) {
                const int rows = dir == 0 ? nn : nt, NR = 16 * ((rows + 15) / 16);
                off[2 * (p * (kMaxOrder + 1) + m) + dir] = (int)tab.size();
                const size_t base = tab.size();
                tab.resize(base + (size_t)nch * NR * kK, 0.f);
                for (int r = 0; r < rows; ++r)
                    for (int k = 0; k < 3 * nt; ++k) {
                        const int b = k / nt, q = k - b * nt;
                        int j, n;
                        if (dir == 0) {
                            n = m + r;
                            j = q;
                        } else {
                            j = r;
                            n = m + q;
                            if (n > p) continue;
                        }
                        const int id = cidx(n, m);
                        double v = b == 0 ? T.P[j * nc + id] : (b == 1 ? T.dP[j * nc + id] : m * T.Ps[j * nc + id]);
                        if (dir == 0) v *= T.wq[j];
                        tab[base + (size_t)(k / kK) * NR * kK + kmaj(r, k % kK)] = float(v);
                    }
            }
        }
    }
    c->n_leg_tiles = (int)tiles.size();
    c->d_leg_tiles.upload(tiles);
    c->d_leg_sph.upload(sph);
    c->d_leg_tab.upload(tab);
    c->d_leg_off.upload(off);
    const long long stride = 6LL * (c->pmax + 1) * (c->pmax + 1);
    c->d_fgbuf.alloc(sizeof(float) * stride * std::max(c->N, 1));
    c->d_lopbuf.alloc(sizeof(double) * 6 * std::max(c->N, 1));
}

// device pointers and sizes of the geometry, as the kernels receive them
// Coarse levels of every sphere for this geometry and one tolerance: for each far pair (t, s) of a
// problem the coarsest ladder order pe < p_s with pe >= log(eps) / log(a_s / r_min) + margin,
// r_min = |c_t - c_s| - a_t (s as the source; the kernels use the coarsest level built that satisfies
// it) and, with coarse targets, the same with the target margin for s as the target of t (if that
// level has at most kCoarseTargetNum / kCoarseTargetDen of s's grid points); at most kCoarseLevels
// orders per sphere (the finest kept). Maps (and their transposes) are shared per (p, pe). Then the
// coarse-target entries, their candidates, work items and interpolation tiles.
// x rounded to TF32 (10 explicit mantissa bits; to nearest, ties away from zero), as cvt.rna.tf32 does
float tf32_rna_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}

// Workspace of the tensor-core strengths (FP32 set), only while they are selected: the split partials
// (kCoarseTcSplit x the coarse points) and the per-tile counters, zeroed once (the kernel leaves them zero).
void coarse_tc_buffers(smob_ctx* c, smob_ctx::CoarseHost& h) {
    if (!c->coarse_tc || h.hp) return;
    h.d_cpart.alloc(sizeof(float4) * (size_t)kCoarseTcSplit * (size_t)std::max(h.ncoarse, 1));
    h.d_ctile_count.alloc(sizeof(unsigned) * std::max<size_t>(h.cdesc_tc.size(), 1));
    CUDA_OK(cudaMemsetAsync(h.d_ctile_count.p, 0, h.d_ctile_count.bytes, c->st));
}

// Nodes of an entry's next far-field work block with rem nodes left: the cap while rem fills it, else
// a power of two from floor up, taken whole if rem fills at least 3/4 of it (one CTA with a few idle
// nodes), else its half (a full block; the rest in smaller ones).
int ct_block_nodes(int rem, int cap, int floor) {
    if (rem >= cap) return cap;
    int hi = floor;
    while (hi < rem) hi <<= 1;
    return (hi == floor || 4 * rem >= 3 * hi) ? hi : hi >> 1;
}

void build_coarse_set(smob_ctx* c, smob_ctx::CoarseHost& h, std::vector<double>& nodes, std::vector<int>& node_off,
                      std::vector<char>& have_nodes) {
    const int N = c->N;
    h.clev.assign((size_t)N * kCoarseLevels, make_int4(0, 0, 0, 0));
    h.cent.clear();
    h.ncoarse = 0;
    std::vector<float> maps, mapsT;
    std::vector<double> mapsd, mapsTd;
    std::map<int, int> map_off;  // p * 64 + pe -> offset in the maps
    if (h.eps > 0) {
        const double leps = std::log(h.eps);
        for (int pi = 0; pi < c->P; ++pi) {
            const Problem& pr = c->problems[pi];
            for (int s = pr.s0; s < pr.s1; ++s) {
                const int ps = c->orders[s];
                const double as = c->radii[s];
                std::vector<char> used(sizeof(kCoarseLadder) / sizeof(int), 0);
                for (int t = pr.s0; t < pr.s1; ++t) {
                    if (t == s) continue;
                    double d2 = 0;
                    for (int k = 0; k < 3; ++k) {
                        const double dk = c->centers[3 * t + k] - c->centers[3 * s + k];
                        d2 += dk * dk;
                    }
                    const double d = std::sqrt(d2);
                    if (d < 1.5 * (as + c->radii[t])) continue;  // near pair: spectral, not far field
                    const double rmin = d - c->radii[t];
                    if (!(rmin > as)) continue;
                    const double need = leps / std::log(as / rmin) + kCoarseMargin;
                    for (size_t l = 0; l < used.size(); ++l)
                        if (kCoarseLadder[l] >= need) {
                            if (kCoarseLadder[l] < ps) used[l] = 1;
                            break;
                        }
                    // s as the target of t: the same ratio a_s / (|c_t - c_s| - a_t), its own margin,
                    // and a level only if it has at most kCoarseTargetNum / kCoarseTargetDen of the grid
                    if (h.ctgt) {
                        const double need_t = leps / std::log(as / rmin) + kCoarseTargetMargin;
                        for (size_t l = 0; l < used.size(); ++l)
                            if (kCoarseLadder[l] >= need_t) {
                                const int pe = kCoarseLadder[l];
                                if (pe < ps && (pe + 1) * (2 * pe + 2) * kCoarseTargetDen <= c->glen[s] * kCoarseTargetNum)
                                    used[l] = 1;
                                break;
                            }
                    }
                }
                std::vector<int> pes;
                for (size_t l = 0; l < used.size(); ++l)
                    if (used[l]) pes.push_back(kCoarseLadder[l]);
                if ((int)pes.size() > kCoarseLevels) pes.erase(pes.begin(), pes.end() - kCoarseLevels);
                for (int l = 0; l < (int)pes.size(); ++l) {
                    const int pe = pes[l];
                    const int key = ps * 64 + pe;
                    if (!map_off.count(key)) {
                        // the map [fine j][coarse k] and, at the same offset, its transpose [k][j]
                        // (the coarse targets' interpolation)
                        const int ngf = (ps + 1) * (2 * ps + 2), nec = (pe + 1) * (2 * pe + 2);
                        if (h.hp) {
                            const std::vector<double>& m = coarse_map_d(ps, pe);
                            map_off[key] = (int)mapsd.size();
                            mapsd.insert(mapsd.end(), m.begin(), m.end());
                            mapsTd.resize(mapsd.size());
                            for (int j = 0; j < ngf; ++j)
                                for (int k = 0; k < nec; ++k)
                                    mapsTd[map_off[key] + (size_t)k * ngf + j] = m[(size_t)j * nec + k];
                        } else {
                            const std::vector<float>& m = coarse_map(ps, pe);
                            map_off[key] = (int)maps.size();
                            maps.insert(maps.end(), m.begin(), m.end());
                            mapsT.resize(maps.size());
                            for (int j = 0; j < ngf; ++j)
                                for (int k = 0; k < nec; ++k)
                                    mapsT[map_off[key] + (size_t)k * ngf + j] = m[(size_t)j * nec + k];
                        }
                    }
                    if (!have_nodes[pe]) {
                        std::vector<double> nv;
                        unit_nodes(pe, nv);
                        node_off[pe] = (int)(nodes.size() / 3);
                        nodes.insert(nodes.end(), nv.begin(), nv.end());
                        have_nodes[pe] = 1;
                    }
                    const int cnt = (pe + 1) * (2 * pe + 2);
                    h.clev[(size_t)s * kCoarseLevels + l] = make_int4(pe, h.ncoarse, cnt, map_off[key]);
                    h.cent.push_back(make_int2(s, l));
                    h.ncoarse += cnt;
                }
            }
        }
    }
    // GEMM tiles of the per-pass strengths: entries grouped by map (p, pe), 8 spheres x kCoarseTileNodes
    // coarse nodes per CTA
    h.cdesc.clear();
    h.cdesc_tc.clear();
    h.cgrp.clear();
    h.gent.clear();
    struct MapGroup {
        int ng = 0, cnt = 0;
        std::vector<int2> ents;  // {sphere, first coarse point}
    };
    std::map<int, MapGroup> by_map;  // by map offset
    for (const int2& e : h.cent) {
        const int4 L = h.clev[(size_t)e.x * kCoarseLevels + e.y];
        MapGroup& mg = by_map[L.w];
        mg.ng = c->glen[e.x];
        mg.cnt = L.z;
        mg.ents.push_back(make_int2(e.x, L.y));
    }
    for (auto& kv : by_map) {
        const MapGroup& mg = kv.second;
        const int grp = (int)h.cgrp.size();
        h.cgrp.push_back(make_int4(kv.first, mg.ng, mg.cnt, 0));
        const int first = (int)h.gent.size();
        h.gent.insert(h.gent.end(), mg.ents.begin(), mg.ents.end());
        for (int e = 0; e < (int)mg.ents.size(); e += 8)
            for (int k0 = 0; k0 < mg.cnt; k0 += kCoarseTileNodes)
                h.cdesc.push_back(make_int4(grp, k0, first + e, std::min(8, (int)mg.ents.size() - e)));
        if (!h.hp)  // the tensor-core tiles of the FP32 set
            for (int e = 0; e < (int)mg.ents.size(); e += kCoarseTcSph)
                for (int k0 = 0; k0 < mg.cnt; k0 += kCoarseTcNodes)
                    h.cdesc_tc.push_back(
                        make_int4(grp, k0, first + e, std::min(kCoarseTcSph, (int)mg.ents.size() - e)));
    }
    // Coarse targets: for every sphere t and level l small enough to serve as its targets, the source
    // spheres whose pair may take that level (tgt_level on the device, in FP32 from FP32 centres:
    // listed here in FP64 with a margin of kCtRuleSlack orders on both sides of each level boundary,
    // so a pair near a boundary is a candidate of both levels and the device check picks one). Work
    // items: node blocks (ct_block_nodes) x candidate ranges of about kCtSrcPoints source points.
    constexpr double kCtRuleSlack = 1e-3;
    constexpr int kCtSrcPoints = 512;
    h.ctent.clear();
    h.ctsrc.clear();
    h.ct_work.clear();
    h.ctitile.clear();
    h.ctient.clear();
    h.ctitile_tc.clear();
    h.ctient_tc.clear();
    std::vector<float> mapI;  // the interpolation maps' pre-split A tiles (FP32 set)
    std::vector<double> work_cost;
    h.ctused.assign((size_t)std::max(N, 1) * kCoarseLevels, 0);
    h.ct_partial = 0;
    // Built whenever coarse targets are on and the set compresses (eps > 0), also when no sphere of the
    // context has a coarse level (the grid entries alone): which far-field kernel runs must not depend on
    // the data, or a problem would take another kernel (and other bits) alone than in a batch whose
    // other problems have well-separated pairs.
    if (h.ctgt && h.eps > 0) {
        const double leps = std::log(h.eps);
        auto dist = [&](int t, int s) {
            double d2 = 0;
            for (int k = 0; k < 3; ++k) {
                const double dk = c->centers[3 * t + k] - c->centers[3 * s + k];
                d2 += dk * dk;
            }
            return std::sqrt(d2);
        };
        // source points a candidate will likely be read from (its coarse level for t, or its grid)
        auto src_points = [&](int t, int s, double d) {
            const int4* L = &h.clev[(size_t)s * kCoarseLevels];
            const double rmin = d - c->radii[t];
            if (L[0].x != 0 && rmin > c->radii[s]) {
                const double need = leps / std::log(c->radii[s] / rmin) + kCoarseMargin;
                for (int l = 0; l < kCoarseLevels && L[l].x != 0; ++l)
                    if (L[l].x >= need) return L[l].z;
            }
            return c->glen[s];
        };
        // slot kCoarseLevels: the grid entry's candidates (pairs that stay on the grid targets)
        std::vector<std::vector<int>> cand(kCoarseLevels + 1), pts(kCoarseLevels + 1);
        auto add_entry = [&](int t, int l, int q0, int n, int pi) {
            const int slot = l < 0 ? kCoarseLevels : l;
            CtEnt e{};
            e.t = t;
            e.l = l;
            e.q0 = q0;
            e.n = n;
            e.src0 = (int)h.ctsrc.size();
            e.nsrc = (int)cand[slot].size();
            e.problem = pi;
            e.poff = h.ct_partial;
            std::vector<std::pair<int, int>> chunks;
            std::vector<int> chunk_pts;
            for (int a = 0, acc = 0, i = 0; i < e.nsrc; ++i) {
                acc += pts[slot][i];
                if (acc >= kCtSrcPoints || i + 1 == e.nsrc) {
                    chunks.push_back({e.src0 + a, e.src0 + i + 1});
                    chunk_pts.push_back(acc);
                    a = i + 1;
                    acc = 0;
                }
            }
            e.nchunks = (int)chunks.size();  // 0: no candidates, the sums are zeros
            h.ct_partial += (h.hp ? 6LL : 3LL) * e.n * e.nchunks;
            h.ctsrc.insert(h.ctsrc.end(), cand[slot].begin(), cand[slot].end());
            const int ei = (int)h.ctent.size();
            h.ctent.push_back(e);
            if (l >= 0) h.ctused[(size_t)t * kCoarseLevels + l] = 1;
            for (int k0 = 0, rem = e.n; rem > 0 && e.nchunks > 0;) {
                // FP32: blocks of 128 ... 8 nodes on kFarThreads threads; float-float: 64 ... 4 nodes
                // (two per thread of kFarThreadsDF); the rest of the CTA takes slices of the sources
                const int w = h.hp ? ct_block_nodes(rem, 2 * kFarThreadsDF, 4) : ct_block_nodes(rem, kFarThreads, 8);
                const int nb = std::min(w, rem);
                for (int ci = 0; ci < e.nchunks; ++ci) {
                    h.ct_work.push_back(CtWork{ei, k0, nb, w, chunks[ci].first, chunks[ci].second, ci, 0});
                    // the CTA's time: its source points over its slices
                    work_cost.push_back((double)chunk_pts[ci] * w / kFarThreads);
                }
                k0 += nb;
                rem -= nb;
            }
        };
        for (int pi = 0; pi < c->P; ++pi) {
            const Problem& pr = c->problems[pi];
            for (int t = pr.s0; t < pr.s1; ++t) {
                const int4* L = &h.clev[(size_t)t * kCoarseLevels];
                for (auto& v : cand) v.clear();
                for (auto& v : pts) v.clear();
                for (int s = pr.s0; s < pr.s1; ++s) {
                    if (s == t) continue;
                    bool nearp = false;
                    for (int e = c->nbr_start[t]; e < c->nbr_start[t + 1] && !nearp; ++e) nearp = c->nbr_src[e] == s;
                    if (nearp) continue;
                    const double d = dist(t, s);
                    const double rmin = d - c->radii[s];
                    // the grid entry keeps every pair not certainly taken by one coarse-target level
                    bool certain = false;
                    if (L[0].x != 0 && rmin > c->radii[t]) {
                        const double need = leps / std::log(c->radii[t] / rmin) + kCoarseTargetMargin;
                        for (int l = 0; l < kCoarseLevels && L[l].x != 0; ++l) {
                            if (L[l].z * kCoarseTargetDen > c->glen[t] * kCoarseTargetNum) break;  // and every finer
                            if (L[l].x >= need - kCtRuleSlack && (l == 0 || L[l - 1].x < need + kCtRuleSlack)) {
                                cand[l].push_back(s);
                                pts[l].push_back(src_points(t, s, d));
                                if (L[l].x >= need + kCtRuleSlack && (l == 0 || L[l - 1].x < need - kCtRuleSlack))
                                    certain = true;
                            }
                        }
                    }
                    if (!certain) {
                        cand[kCoarseLevels].push_back(s);
                        pts[kCoarseLevels].push_back(src_points(t, s, d));
                    }
                }
                add_entry(t, -1, c->gidx[t], c->glen[t], pi);
                for (int l = 0; l < kCoarseLevels; ++l)
                    if (!cand[l].empty()) add_entry(t, l, L[l].y, L[l].z, pi);
            }
        }
        // longest items first (the tail of the one wave they usually fill)
        std::vector<int> order(h.ct_work.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work_cost[a] > work_cost[b]; });
        std::vector<CtWork> sorted(order.size());
        for (size_t i = 0; i < order.size(); ++i) sorted[i] = h.ct_work[order[i]];
        h.ct_work.swap(sorted);
        // interpolation tiles: listed entries grouped by map, 2 entries x 128 grid points (float-float: 1 x 256)
        std::map<int, std::vector<int>> by_map;
        for (int i = 0; i < (int)h.ctent.size(); ++i) {
            const CtEnt& e = h.ctent[i];
            if (e.l >= 0) by_map[h.clev[(size_t)e.t * kCoarseLevels + e.l].w].push_back(i);
        }
        for (auto& kv : by_map) {
            const CtEnt& e0 = h.ctent[kv.second[0]];
            const int ng = c->glen[e0.t], n = e0.n;
            const size_t per = h.hp ? kCiEntD : kCiEnt;  // entries per tile (what the kernels read)
            const int pts = h.hp ? kCiPtsD : kCiPts;        // grid points per tile
            for (size_t a = 0; a < kv.second.size(); a += per) {
                const int first = (int)h.ctient.size();
                const int ne = (int)std::min<size_t>(per, kv.second.size() - a);
                h.ctient.insert(h.ctient.end(), kv.second.begin() + a, kv.second.begin() + a + ne);
                for (int j0 = 0; j0 < ng; j0 += pts) h.ctitile.push_back(CtITile{kv.first, ng, n, first, ne, j0, 0, 0});
            }
            if (h.hp) continue;
            // the same entries for the tensor-core kernel: 16 per tile, A = the map [grid point][coarse
            // node] in tiles of 128 grid points x 32 coarse nodes, split into TF32 hi and lo (rounded to
            // nearest) in the MMA's core-matrix order
            const int nmt = (ng + kCoarseTcNodes - 1) / kCoarseTcNodes, nck = (n + 31) / 32;
            const int aoff = (int)mapI.size();
            mapI.resize(mapI.size() + (size_t)nmt * nck * 2 * kCoarseTcNodes * 32, 0.f);
            for (int mt = 0; mt < nmt; ++mt)
                for (int ch = 0; ch < nck; ++ch) {
                    float* hi = &mapI[(size_t)aoff + (size_t)(mt * nck + ch) * 2 * kCoarseTcNodes * 32];
                    float* lo = hi + kCoarseTcNodes * 32;
                    for (int r = 0; r < kCoarseTcNodes; ++r)
                        for (int k = 0; k < 32; ++k) {
                            const int j = mt * kCoarseTcNodes + r, kk = ch * 32 + k;
                            const float v = (j < ng && kk < n) ? maps[(size_t)kv.first + (size_t)j * n + kk] : 0.f;
                            const float vh = tf32_rna_host(v);
                            const size_t o = tc::kmajor_offset(r, k, 32) / 4;
                            hi[o] = vh;
                            lo[o] = tf32_rna_host(v - vh);
                        }
                }
            for (size_t a = 0; a < kv.second.size(); a += kCoarseTcSph) {
                const int first = (int)h.ctient_tc.size();
                const int ne = (int)std::min<size_t>(kCoarseTcSph, kv.second.size() - a);
                h.ctient_tc.insert(h.ctient_tc.end(), kv.second.begin() + a, kv.second.begin() + a + ne);
                for (int j0 = 0; j0 < ng; j0 += kCoarseTcNodes)
                    h.ctitile_tc.push_back(CtITile{aoff, ng, n, first, ne, j0, 0, 0});
            }
        }
    }
    h.d_clev.upload(h.clev);
    h.d_cent.upload(h.cent);
    h.d_cdesc.upload(h.cdesc);
    h.d_cdesc_tc.upload(h.cdesc_tc);
    h.d_cgrp.upload(h.cgrp);
    h.d_gent.upload(h.gent);
    if (h.hp) {
        // the float-float strength GEMM's maps as (hi, lo) float pairs
        std::vector<float2> mapsf2(mapsd.size());
        for (size_t i = 0; i < mapsd.size(); ++i) {
            const float hi = float(mapsd[i]);
            mapsf2[i] = make_float2(hi, float(mapsd[i] - double(hi)));
        }
        h.d_cmap.upload(mapsf2);
    } else {
        h.d_cmap.upload(maps);
    }
    if (!h.hp) {
        // The tensor-core strength GEMM's A operand, prepared once per geometry: per map group, per M
        // tile of 128 coarse nodes and K chunk of 32 fine nodes, the transposed map's block split into
        // TF32 high and low parts (both rounded to nearest, ties away), each 16 KB in the MMA's K-major
        // core-matrix order, so a CTA stages it with straight coalesced copies. cgrp.w: its offset.
        std::vector<float> mapA;
        for (int4& G : h.cgrp) {
            const int ng = G.y, cnt = G.z, nmt = (cnt + kCoarseTcNodes - 1) / kCoarseTcNodes, nck = (ng + 31) / 32;
            G.w = (int)mapA.size();
            mapA.resize(mapA.size() + (size_t)nmt * nck * 2 * kCoarseTcNodes * 32, 0.f);
            for (int mt = 0; mt < nmt; ++mt)
                for (int ch = 0; ch < nck; ++ch) {
                    float* hi = &mapA[(size_t)G.w + (size_t)(mt * nck + ch) * 2 * kCoarseTcNodes * 32];
                    float* lo = hi + kCoarseTcNodes * 32;
                    for (int r = 0; r < kCoarseTcNodes; ++r)
                        for (int k = 0; k < 32; ++k) {
                            const int kk = mt * kCoarseTcNodes + r, j = ch * 32 + k;
                            const float v = (kk < cnt && j < ng) ? mapsT[(size_t)G.x + (size_t)kk * ng + j] : 0.f;
                            const float vh = tf32_rna_host(v);
                            const size_t o = tc::kmajor_offset(r, k, 32) / 4;
                            hi[o] = vh;
                            lo[o] = tf32_rna_host(v - vh);
                        }
                }
        }
        h.d_cmapA.upload(mapA);
        h.d_cgrp.upload(h.cgrp);  // with the offsets
        coarse_tc_buffers(c, h);
    }
    const size_t np = std::max(h.ncoarse, 1);
    h.d_cpos32.alloc(sizeof(float4) * np);
    if (h.hp) h.d_cpos32lo.alloc(sizeof(float4) * np);
    h.d_csrc.alloc(sizeof(float4) * np * (h.hp ? 2 : 1));
    if (!h.ctent.empty()) {
        h.d_ctent.upload(h.ctent);
        h.d_ctsrc.upload(h.ctsrc);
        h.d_ctcand.alloc(sizeof(int2) * std::max<size_t>(h.ctsrc.size(), 1));
        h.d_ctused.upload(h.ctused);
        h.d_ct_work.upload(h.ct_work);
        h.d_ctitile.upload(h.ctitile);
        h.d_ctient.upload(h.ctient);
        if (!h.hp) {
            h.d_ctitile_tc.upload(h.ctitile_tc);
            h.d_ctient_tc.upload(h.ctient_tc);
            h.d_cmapI.upload(mapI);
        }
        const size_t slots = (size_t)(kCoarseLevels + 1) * (size_t)std::max(c->M, 1);
        h.d_cnrm32.alloc(sizeof(float4) * np);
        if (h.hp) {
            h.d_ct_partial.alloc(sizeof(double) * (size_t)h.ct_partial);
            h.d_ctinterp.alloc(sizeof(double) * 6 * slots);
            // (hi, lo) float pairs of the FP64 transposed maps (the float-float interpolation)
            std::vector<float2> mapsTdf(mapsTd.size());
            for (size_t i = 0; i < mapsTd.size(); ++i) {
                const float hi = float(mapsTd[i]);
                mapsTdf[i] = make_float2(hi, float(mapsTd[i] - double(hi)));
            }
            h.d_cmapT.upload(mapsTdf);
            h.d_cnrm32lo.alloc(sizeof(float4) * np);
            h.d_ctu.alloc(sizeof(double) * 6 * np);
        } else {
            h.d_ct_partial.alloc(sizeof(float) * (size_t)h.ct_partial);
            h.d_ctinterp.alloc(sizeof(float) * 3 * slots);
            h.d_ctu.alloc(sizeof(float4) * np);
        }
    }
    // FP32 set: the transposed maps serve the coarse targets' interpolation and the tensor-core
    // strength GEMM (its A operand), so they are kept with or without coarse targets
    if (!h.hp) h.d_cmapT.upload(mapsT);
}

void build_coarse(smob_ctx* c) {
    std::vector<double> nodes;
    std::vector<int> node_off(kMaxOrder + 1, 0);
    std::vector<char> have_nodes(kMaxOrder + 1, 0);
    build_coarse_set(c, c->c32, nodes, node_off, have_nodes);
    build_coarse_set(c, c->chp, nodes, node_off, have_nodes);
    c->d_cnode.upload(nodes);
    c->d_cnode_off.upload(node_off);
    // sphere centres relative to their problem's origin and radii, FP32, for the kernels' level votes
    std::vector<float4> sph(c->N);
    for (int i = 0; i < c->N; ++i) {
        const double* o = &c->org[3 * c->prob[i]];
        sph[i] = make_float4(float(c->centers[3 * i] - o[0]), float(c->centers[3 * i + 1] - o[1]),
                             float(c->centers[3 * i + 2] - o[2]), float(c->radii[i]));
    }
    c->d_sph32.upload(sph);
}

// coarse points of both sets (after the grid; geometry-dependent)
void coarse_grids(smob_ctx* c) {
    check_launch(c, launch_coarse_grid(c->g, c->g.cs32, c->d_org.as<double>(), c->c32.d_cpos32.as<float4>(), nullptr,
                                       c->c32.ctent.empty() ? nullptr : c->c32.d_cnrm32.as<float4>(), nullptr,
                                       c->st));
    const bool hpct = !c->chp.ctent.empty();
    check_launch(c, launch_coarse_grid(c->g, c->g.cshp, c->d_org.as<double>(), c->chp.d_cpos32.as<float4>(),
                                       c->chp.d_cpos32lo.as<float4>(), hpct ? c->chp.d_cnrm32.as<float4>() : nullptr,
                                       hpct ? c->chp.d_cnrm32lo.as<float4>() : nullptr, c->st));
    // the coarse-target candidates of this geometry
    check_launch(c, launch_ct_classify(c->g, c->g.cs32, c->st));
    check_launch(c, launch_ct_classify(c->g, c->g.cshp, c->st));
}

void bind_geom(smob_ctx* c) {
    DevGeom& g = c->g;
    g.N = c->N;
    g.M = c->M;
    g.P = c->P;
    g.pmax = c->pmax;
    g.center = c->d_center.as<double>();
    g.radius = c->d_radius.as<double>();
    g.quat = c->d_quat.as<double>();
    g.order = c->d_order.as<int>();
    g.gidx = c->d_gidx.as<int>();
    g.glen = c->d_glen.as<int>();
    g.coff = c->d_coff.as<int>();
    g.prob = c->d_prob.as<int>();
    g.coords = c->d_coords.as<double>();
    g.norms = c->d_norms.as<double>();
    g.weights = c->d_weights.as<double>();
    g.sid = c->d_sid.as<int>();
    g.pos32 = c->d_pos32.as<float4>();
    g.nrm32 = c->d_nrm32.as<float4>();
    g.pos32lo = c->d_pos32lo.as<float4>();
    g.nrm32lo = c->d_nrm32lo.as<float4>();
    g.pos64 = c->d_pos64.as<double4_32a>();
    g.nrm64 = c->d_nrm64.as<double4_32a>();
    g.nbr_start = c->d_nbr_start.as<int>();
    g.nbr_src = c->d_nbr_src.as<int>();
    g.nbr_precise = c->d_nbr_precise.as<unsigned char>();
    g.near_src_slot = c->d_near_slot.as<int>();
    g.problems = c->d_problems.as<Problem>();
    g.tabs = c->d_tabs.as<OrderTables>();
    g.tab_d = c->d_tab_d.as<double>();
    g.tab_f = c->d_tab_f.as<float>();
    g.map_rowptr = c->d_map_rowptr.as<int>();
    g.map_col = c->d_map_col.as<int>();
    g.map_val_d = c->d_map_val_d.as<double>();
    g.map_val_f = c->d_map_val_f.as<float>();
    g.active = c->d_active.as<unsigned char>();
    g.near_tc = c->near_tc ? 1 : 0;
    g.coarse_tc = c->coarse_interp_tc ? 1 : 0;
    g.err = c->d_err.as<int>();
    g.sph_tc = c->sph_tc ? 1 : 0;
    g.n_leg_tiles = c->n_leg_tiles;
    g.leg_tiles = c->d_leg_tiles.as<int4>();
    g.leg_sph = c->d_leg_sph.as<int>();
    g.leg_tab = c->d_leg_tab.as<float>();
    g.leg_off = c->d_leg_off.as<int>();
    g.fgbuf = c->d_fgbuf.as<float>();
    g.fg_stride = 6LL * (c->pmax + 1) * (c->pmax + 1);
    g.lopbuf = c->d_lopbuf.as<double>();
    auto bind_set = [&](const smob_ctx::CoarseHost& h, CoarseSet& cs) {
        cs.ncent = (int)h.cent.size();
        cs.clog_eps = h.eps > 0 ? float(std::log(h.eps)) : 0.f;
        cs.cmargin = float(kCoarseMargin);
        cs.clev = h.d_clev.as<int4>();
        cs.cent = h.d_cent.as<int2>();
        cs.cpos32 = h.d_cpos32.as<float4>();
        cs.cpos32lo = h.hp ? h.d_cpos32lo.as<float4>() : nullptr;
        cs.cmap = h.hp ? nullptr : h.d_cmap.as<float>();
        cs.cmapf2 = h.hp ? h.d_cmap.as<float2>() : nullptr;
        cs.csrc = h.d_csrc.as<float4>();
        cs.crep = c->nrep > 1 ? h.ncoarse / c->nrep : h.ncoarse;
        cs.ncdesc = (int)h.cdesc.size();
        cs.cdesc = h.d_cdesc.as<int4>();
        cs.ncdesc_tc = (int)h.cdesc_tc.size();
        cs.cdesc_tc = h.d_cdesc_tc.as<int4>();
        cs.cmapA = h.hp ? nullptr : h.d_cmapA.as<float4>();
        cs.cpart = h.d_cpart.as<float4>();
        cs.ctile_count = h.d_ctile_count.as<unsigned>();
        cs.ncoarse32 = h.ncoarse;
        cs.cgrp = h.d_cgrp.as<int4>();
        cs.gent = h.d_gent.as<int2>();
        const bool ct = !h.ctent.empty();
        cs.ctgt = ct ? 1 : 0;
        cs.ctmargin = float(kCoarseTargetMargin);
        cs.cnrm32 = ct ? h.d_cnrm32.as<float4>() : nullptr;
        cs.cnrm32lo = ct && h.hp ? h.d_cnrm32lo.as<float4>() : nullptr;
        cs.cmapT = !h.hp && h.d_cmapT.p ? h.d_cmapT.as<float>() : nullptr;
        cs.cmapTdf = ct && h.hp ? h.d_cmapT.as<float2>() : nullptr;
        cs.ctused = ct ? h.d_ctused.as<int>() : nullptr;
        cs.nctent = ct ? (int)h.ctent.size() : 0;
        cs.ctent = ct ? h.d_ctent.as<CtEnt>() : nullptr;
        cs.ctsrc = ct ? h.d_ctsrc.as<int>() : nullptr;
        cs.ctcand = ct ? h.d_ctcand.as<int2>() : nullptr;
        cs.ctinterp = ct && !h.hp ? h.d_ctinterp.as<float>() : nullptr;
        cs.ctinterpd = ct && h.hp ? h.d_ctinterp.as<double>() : nullptr;
        cs.nctitile_tc = ct && !h.hp ? (int)h.ctitile_tc.size() : 0;
        cs.ctitile_tc = ct && !h.hp ? h.d_ctitile_tc.as<CtITile>() : nullptr;
        cs.ctient_tc = ct && !h.hp ? h.d_ctient_tc.as<int>() : nullptr;
        cs.cmapI = ct && !h.hp ? h.d_cmapI.as<float4>() : nullptr;
        cs.nctitile = ct ? (int)h.ctitile.size() : 0;
        cs.ctitile = ct ? h.d_ctitile.as<CtITile>() : nullptr;
        cs.ctient = ct ? h.d_ctient.as<int>() : nullptr;
        cs.ctu = ct && !h.hp ? h.d_ctu.as<float4>() : nullptr;
        cs.ctud = ct && h.hp ? h.d_ctu.as<double>() : nullptr;
    };
    bind_set(c->c32, g.cs32);
    bind_set(c->chp, g.cshp);
    g.cnode = c->d_cnode.as<double>();
    g.cnode_off = c->d_cnode_off.as<int>();
    g.sph32 = c->d_sph32.as<float4>();
}

// the FP32 coarse strengths of the current sources: tensor cores or the SIMT GEMM
int coarse_src(smob_ctx* c, cudaStream_t st) {
    return c->coarse_tc ? launch_coarse_src_tc(c->g, c->d_src32.as<float4>(), st)
                        : launch_coarse_src(c->g, c->d_src32.as<float4>(), st);
}

// Tile-shape autotuner: times the FP32 traction far field with 1, 2 and 4 targets per thread on
// this context's geometry (CUDA events, best of two) and keeps the fastest. Results are cached per
// (largest order, size bucket of M) for the process, so contexts of similar shape reuse them.
void autotune_far32(smob_ctx* c) {
    static std::mutex mu;
    static std::map<long long, int> cache;
    const long long key = (long long)c->pmax * 1000 + (long long)std::floor(2.0 * std::log2(double(std::max(c->M, 1))));
    int best = -1;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) best = it->second;
    }
    if (best < 0) {
        cudaEvent_t a, b;
        CUDA_OK(cudaEventCreate(&a));
        CUDA_OK(cudaEventCreate(&b));
        CUDA_OK(cudaMemsetAsync(c->d_src32.p, 0, sizeof(float4) * c->M, c->st));
        check_launch(c, coarse_src(c, c->st));
        DBuf items[3];
        for (int k = 0; k < 3; ++k) items[k].upload(c->items_tpt[k]);
        auto run = [&](int k) {
            check_launch(c, launch_far_field(c->g, items[k].as<FarItem>(), (int)c->items_tpt[k].size(), true, true,
                                             c->d_src32.as<float4>(), nullptr, c->d_partial32.p, c->st, 1 << k));
        };
        auto timed = [&](int k) {
            CUDA_OK(cudaEventRecord(a, c->st));
            run(k);
            CUDA_OK(cudaEventRecord(b, c->st));
            CUDA_OK(cudaEventSynchronize(b));
            float f = 0;
            CUDA_OK(cudaEventElapsedTime(&f, a, b));
            return double(f);
        };
        // Warm up until ~30 ms of far-field work ran (the SM clock ramps up from idle during
        // set-up), then time the variants interleaved round by round so clock drift hits all
        // three alike; the minimum per variant decides.
        double warm = 0;
        for (int i = 0; i < 64 && warm < 30.0; ++i) warm += timed(i % 3);
        const int rounds = warm / 3 < 20.0 ? 4 : 1;
        for (int k = 0; k < 3; ++k) c->tune_ms[k] = 1e300;
        for (int r = 0; r < rounds; ++r)
            for (int k = 0; k < 3; ++k) c->tune_ms[k] = std::min(c->tune_ms[k], timed(k));
        double bestms = 1e300;
        for (int k = 0; k < 3; ++k)
            if (c->tune_ms[k] < bestms) {
                bestms = c->tune_ms[k];
                best = k;
            }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = best;
    } else {
        c->tune_cached = true;
    }
    c->tpt = 1 << best;
    c->items32 = c->items_tpt[best];
    c->d_items32.upload(c->items32);
}

void set_active(smob_ctx* c, const std::vector<unsigned char>& act) { h2d(c, c->d_active.p, act.data(), act.size()); }

// ---------------------------------------------------------------- the operator
// operator precisions: every kernel in FP64; every kernel in FP32; or FP64 sphere and near
// kernels with the far field in float-float (the high-precision operator of the mixed solve)
enum OpPrec { OP_FP64 = 0, OP_FP32 = 1, OP_DF = 2 };

// the fused float-float pass with the float-float set's coarse targets (after its coarse strengths)
bool far_df_ct_on(const smob_ctx* c) { return c->nrep == 1 && !c->chp.ctent.empty(); }
void far_df_ct(smob_ctx* c, cudaStream_t st) {
    check_launch(c, launch_far_df_ct(c->g, c->chp.d_ct_work.as<CtWork>(), (int)c->chp.ct_work.size(),
                                     c->d_srcdf.as<float4>(), c->chp.d_ct_partial.as<double>(), st));
}

// FP32 far field with coarse targets: the listed and grid entries (after the pass's coarse strengths,
// on the far stream); replaces launch_far_field for FP32 passes when the set has entries
bool far_ct_on(const smob_ctx* c) { return !c->c32.ctent.empty(); }
void far_ct(smob_ctx* c, bool trac, cudaStream_t st) {
    ProfScope ps(c, trac ? "far_trac_fp32" : "far_sl_fp32", st);
    check_launch(c, launch_far_ct(c->g, c->c32.d_ct_work.as<CtWork>(), (int)c->c32.ct_work.size(), trac,
                                  c->d_src32.as<float4>(), c->c32.d_ct_partial.as<float>(), st));
}

// The FP32 grid kernels' tile is tuned when a context first runs them: with coarse targets on, its
// FP32 passes use the entry kernel instead and need no tuning.
// Tile tuning of the FP32 grid kernels, run when a context first needs them: at creation, and
// lazily at the next solve or operator call after a geometry or tolerance change left the FP32
// passes without coarse targets (so that an update never runs the ~30 ms timed warm-up itself and
// stays all-or-nothing). The choice is cached per (largest order, size bucket) for the process.
void ensure_tuned(smob_ctx* c) {
    if (c->tuned || far_ct_on(c)) return;
    AllocStreamScope scope(c->st);  // the tuner's item lists live on the context's stream
    autotune_far32(c);
    c->tuned = true;
}

// out (device) += c_id*x + c_sl*S[x] + c_trac*K[x] + c_lop*L[x] on active problems
void op_apply(smob_ctx* c, const double* x, double* out, double c_id, double c_sl, double c_trac, double c_lop,
              int prec) {
    const DevGeom& g = c->g;
    const bool fp32 = prec == OP_FP32, dfar = prec == OP_DF;
    const bool trac = std::fabs(c_trac) > 1e-9, sl = std::fabs(c_sl) > 1e-9;
    const bool id = std::fabs(c_id) > 1e-9;
    void* coef = fp32 ? c->d_coef32.p : c->d_coef64.p;
    void* sets = fp32 ? c->d_sets32.p : c->d_sets64.p;
    void* partial = fp32 ? c->d_partial32.p : c->d_partial64.p;
    const int nslots = (int)c->slot_sphere.size();
    const FarItem* items = fp32 ? c->d_items32.as<FarItem>() : c->d_items64.as<FarItem>();
    const int nitems = (int)(fp32 ? c->items32.size() : c->items64.size());
    auto kind_pass = [&](bool tr, double cc, bool with_id_lop) {
        PassFork fork(c);
        const cudaStream_t fs = fork.far();
        // far field: side stream
        if (dfar) {
            {
                ProfScope ps(c, "far_pack", fs);
                check_launch(c, launch_far_pack_df(g, x, cc, c->d_srcdf.as<float4>(), fs));
                check_launch(c, launch_coarse_src_df(g, c->d_srcdf.as<float4>(), fs));
            }
            ProfScope ps(c, tr ? "far_trac_df" : "far_sl_df", fs);
            check_launch(c, launch_far_field_df(g, c->d_items_df.as<FarItem>(), (int)c->items_df.size(), tr ? 1 : 0,
                                                c->d_srcdf.as<float4>(), static_cast<double*>(partial), nullptr, fs));
        } else {
            {
                ProfScope ps(c, "far_pack", fs);
                check_launch(c, launch_far_pack(g, x, cc, c->d_src32.as<float4>(), c->d_src64.as<double4_32a>(), fp32, fs));
            }
            if (fp32 && g.cs32.ncent > 0) {
                ProfScope ps(c, "far_coarse", fs);
                check_launch(c, coarse_src(c, fs));
            }
            if (fp32 && far_ct_on(c)) {
                far_ct(c, tr, fs);
            } else {
                ProfScope ps(c, fp32 ? (tr ? "far_trac_fp32" : "far_sl_fp32") : (tr ? "far_trac_fp64" : "far_sl_fp64"),
                             fs);
                if (fp32 && c->nrep > 1)
                    check_launch(c, launch_far_field_rep(g, c->d_items_rep.as<FarItem>(), (int)c->items_rep.size(),
                                                         c->nrep, c->rep_M, tr, c->d_src32.as<float4>(),
                                                         static_cast<float*>(partial), fs));
                else
                    check_launch(c, launch_far_field(g, items, nitems, tr, fp32, c->d_src32.as<float4>(),
                                                     c->d_src64.as<double4_32a>(), partial, fs, c->tpt));
            }
        }
        // sphere self and near field: main stream
        {
            ProfScope ps(c, "sphere_self");
            check_launch(c, launch_sphere_op(g, x, out, with_id_lop && id ? c_id : 0.0, cc, tr ? 3 : 0,
                                             with_id_lop ? c_lop : 0.0, coef, fp32, c->st));
        }
        if (nslots > 0) {
            {
                ProfScope ps(c, "near_sets");
                check_launch(c, launch_near_sets(g, coef, tr, fp32, sets, nslots, c->d_slot_sphere.as<int>(),
                                                 tr ? c->set_stride_trac : c->set_stride_sl, c->st, dfar));
            }
            const long long stride = tr ? c->set_stride_trac : c->set_stride_sl;
            {
                // FP32 (tensor cores or SIMT), float-float (the float-float operator) or FP64
                ProfScope ps(c, tr ? "near_eval_trac" : "near_eval_sl");
                check_launch(c, launch_near_eval(g, sets, stride, tr, fp32, cc, out, c->st,
                                                 fp32 && c->n_precise ? 1 : 0, dfar));
            }
            if (fp32 && c->n_precise) {
                // near-singular pairs (gap < 0.1 min radius) in float-float even inside the FP32 operator
                ProfScope ps(c, "near_singular_df");
                check_launch(c, launch_sh_g2s(g, x, c->d_coef64.as<double>(), c->st));
                check_launch(c, launch_near_sets(g, c->d_coef64.p, tr, false, c->d_sets64.p, nslots,
                                                 c->d_slot_sphere.as<int>(), stride, c->st, true));
                check_launch(c, launch_near_eval(g, c->d_sets64.p, stride, tr, false, cc, out, c->st, 2, true));
            }
        }
        fork.join();
        {
            ProfScope ps(c, "far_reduce");
            check_launch(c, launch_far_reduce(g, partial, fp32, tr ? -3.0 / (4 * kPi) : 1.0 / (8 * kPi), out, c->st,
                                              fp32 && far_ct_on(c) ? 1 : 0));
        }
    };
    if (trac) kind_pass(true, c_trac, true);
    if (sl) kind_pass(false, c_sl, !trac);
    if (!trac && !sl && (id || std::fabs(c_lop) > 0)) {
        ProfScope ps(c, "sphere_self");
        check_launch(c, launch_sphere_op(g, x, out, id ? c_id : 0.0, 0.0, -1, c_lop, nullptr, fp32, c->st));
    }
}

// High-precision traction and single layer of one density in one pass, on active problems:
// out_t += c_id*x + c_trac*K[x] and out_s += c_sl*S[x]. Self and near parts in FP64; the far field is
// one float-float pass that evaluates both kernels per pair (shared r, 1/r, r.f).
void op_apply_hp_both(smob_ctx* c, const double* x, double* out_t, double c_id, double c_trac, double* out_s,
                      double c_sl) {
    const DevGeom& g = c->g;
    const int nslots = (int)c->slot_sphere.size();
    c->d_partial64_sl.alloc(sizeof(double) * c->partial64);
    PassFork fork(c);
    const cudaStream_t fs = fork.far();
    {
        ProfScope ps(c, "far_pack", fs);
        check_launch(c, launch_far_pack_df(g, x, 1.0, c->d_srcdf.as<float4>(), fs));
        if (c->nrep == 1) check_launch(c, launch_coarse_src_df(g, c->d_srcdf.as<float4>(), fs));
    }
    const bool hpct = far_df_ct_on(c);
    {
        ProfScope ps(c, "far_both_df", fs);
        if (c->nrep > 1)
            check_launch(c, launch_far_field_df_rep(g, c->d_items_rep.as<FarItem>(), (int)c->items_rep.size(), c->nrep,
                                                    c->rep_M, c->d_srcdf.as<float4>(), c->d_partial64.as<double>(),
                                                    c->d_partial64_sl.as<double>(), fs));
        else if (hpct)
            far_df_ct(c, fs);
        else
            check_launch(c, launch_far_field_df(g, c->d_items_df.as<FarItem>(), (int)c->items_df.size(), 2,
                                                c->d_srcdf.as<float4>(), c->d_partial64.as<double>(),
                                                c->d_partial64_sl.as<double>(), fs));
    }
    {
        ProfScope ps(c, "sphere_self");
        check_launch(c, launch_sphere_op(g, x, out_t, c_id, c_trac, 3, 0.0, c->d_coef64.p, false, c->st));
        check_launch(c, launch_sphere_op(g, x, out_s, 0.0, c_sl, 0, 0.0, nullptr, false, c->st));
    }
    if (nslots > 0) {
        for (int k = 0; k < 2; ++k) {
            const bool tr = k == 0;
            const long long stride = tr ? c->set_stride_trac : c->set_stride_sl;
            {
                ProfScope ps(c, "near_sets");
                check_launch(c, launch_near_sets(g, c->d_coef64.p, tr, false, c->d_sets64.p, nslots,
                                                 c->d_slot_sphere.as<int>(), stride, c->st, true));
            }
            // float-float near field (the FP64 coefficients' sets as float pairs)
            ProfScope ps(c, tr ? "near_eval_trac_df" : "near_eval_sl_df");
            check_launch(c, launch_near_eval(g, c->d_sets64.p, stride, tr, false, tr ? c_trac : c_sl, tr ? out_t : out_s,
                                             c->st, 0, true));
        }
    }
    fork.join();
    ProfScope ps(c, "far_reduce");
    check_launch(c, launch_far_reduce(g, c->d_partial64.p, false, c_trac * (-3.0 / (4 * kPi)), out_t, c->st,
                                      hpct ? 2 : 0));
    check_launch(c, launch_far_reduce(g, c->d_partial64_sl.p, false, c_sl / (8 * kPi), out_s, c->st, hpct ? 3 : 0));
}

// ---------------------------------------------------------------- solver
void ensure_solver(smob_ctx* c, int m) {
    const size_t n = 3 * (size_t)c->M;
    if (m > c->restart_cap) {
        c->drop_graphs();  // captured blocks hold the old buffer addresses
        c->d_V.alloc(sizeof(double) * n * (m + 1));
        c->d_H.alloc(sizeof(double) * c->P * m * (m + 1));
        c->d_g.alloc(sizeof(double) * c->P * (m + 1));
        c->d_cs.alloc(sizeof(double) * c->P * m);
        c->d_sn.alloc(sizeof(double) * c->P * m);
        c->d_y.alloc(sizeof(double) * c->P * m);
        // dots of up to m + 1 vectors per chunk; the fused update-norm step's kElemBlocks per chunk
        c->d_partial_red.alloc(sizeof(double) * c->chunks.size() * std::max(m + 1, kElemBlocks));
        alloc_red_counters(c, m + 1);
        c->restart_cap = m;
    }
    c->d_w.alloc(sizeof(double) * n);
    c->d_r.alloc(sizeof(double) * n);
    c->d_x.alloc(sizeof(double) * n);
    c->d_b.alloc(sizeof(double) * n);
    c->d_rho.alloc(sizeof(double) * n);
    c->d_u.alloc(sizeof(double) * n);
    c->d_force.alloc(sizeof(double) * 6 * c->N);
    c->d_vel.alloc(sizeof(double) * 6 * c->N);
    c->d_kc.alloc(sizeof(int) * c->P);
    c->d_ks.alloc(sizeof(KrylovState) * c->P);
    c->d_norm.alloc(sizeof(double) * c->P);
    c->d_hn.alloc(sizeof(double) * c->P);
    c->d_beta.alloc(sizeof(double) * c->P);
    c->d_incycle.alloc(c->P);
    c->d_track.alloc(sizeof(SolveTrack) * c->P);
    c->d_sparams.alloc(sizeof(SolveParams));
    c->d_updmask.alloc(c->P);
    c->d_hpmask.alloc(c->P);
    c->d_freshmask.alloc(c->P);
    c->d_bnorm.alloc(sizeof(double) * c->P);
    c->d_jdev.alloc(sizeof(int));
    c->d_runs_j.alloc(sizeof(int) * std::max(m, c->restart_cap));
    if (!c->d_xlast.p) {
        c->d_xlast.alloc(sizeof(double) * n);
        CUDA_OK(cudaMemsetAsync(c->d_xlast.p, 0, sizeof(double) * n, c->st));
    }
}

std::vector<double> seg_norms(smob_ctx* c, const double* v, const unsigned char* active) {
    KrylovLaunch L = c->kl();
    check_launch(c, launch_dots(L, v, 0, 1, v, active, c->d_norm.as<double>(), 1, 0, false, true, c->st));
    std::vector<double> h(c->P);
    d2h(c, h.data(), c->d_norm.p, sizeof(double) * c->P);
    return h;
}

// Recycled solutions for a sequence of solves on one geometry (the caller the reference prepares
// for at BIE/SphereSTKMobMat.cpp:232: the collision solver's repeated mobility solves, whose forces
// are combinations of a few contact forces). Every solve with warm_start 2 adds its pair (F, mu),
// A mu = b(F) to the tolerance. The forces are kept orthonormal per problem (classical Gram-Schmidt,
// twice, on the host: 6N values each) and the mu's transformed with the same coefficients on the
// device, so each kept mu column solves the system of its force column. b, rho and mu are linear
// in F, so a new solve starts from mu0 = U h, h = Q^T F: exact (to the tolerance of the earlier
// solves) when F lies in their span, the least-squares fit otherwise. When full, the space starts
// again from the newest pair.

// parts[k] = U_k Q^T F (k < nparts, null parts skipped) on every problem; returns per problem
// |F - Q Q^T F| / |F|
std::vector<double> recycle_guess(smob_ctx* c, const std::vector<double>& f, double* const* parts, int nparts) {
    const size_t n = 3 * (size_t)c->M;
    const size_t n6 = 6 * (size_t)c->N;
    const int P = c->P;
    std::vector<double> h((size_t)P * kRecycleMax, 0.0), fn2(P, 0.0);
    for (int s = 0; s < c->N; ++s) {
        const int p = c->prob[s];
        for (int i = 6 * s; i < 6 * s + 6; ++i) {
            fn2[p] += f[i] * f[i];
            for (int j = 0; j < c->rk; ++j) h[(size_t)p * kRecycleMax + j] += c->rq[n6 * j + i] * f[i];
        }
    }
    // |F - Q h| from the vector itself (|F|^2 - |h|^2 would lose everything below ~1e-8)
    std::vector<double> res2(P, 0.0), est(P, 1.0);
    for (int s = 0; s < c->N; ++s) {
        const int p = c->prob[s];
        for (int i = 6 * s; i < 6 * s + 6; ++i) {
            double e = f[i];
            for (int j = 0; j < c->rk; ++j) e -= h[(size_t)p * kRecycleMax + j] * c->rq[n6 * j + i];
            res2[p] += e * e;
        }
    }
    for (int p = 0; p < P; ++p)
        if (fn2[p] > 0) est[p] = std::sqrt(res2[p] / fn2[p]);
    KrylovLaunch L = c->kl();
    h2d(c, c->d_rcoef.p, h.data(), sizeof(double) * h.size());
    for (int k = 0; k < nparts; ++k) {
        if (!parts[k]) continue;
        CUDA_OK(cudaMemsetAsync(parts[k], 0, sizeof(double) * n, c->st));
        check_launch(c, launch_update(L, c->d_ru.as<double>() + n * k, (long long)(n * kRecycleParts), c->rk, nullptr,
                                      c->d_rcoef.as<double>(), kRecycleMax, 1.0, c->d_active.as<unsigned char>(),
                                      parts[k], c->st));
    }
    CUDA_OK(cudaStreamSynchronize(c->st));  // h must outlive its copy
    return est;
}

// add (F, parts) of the problems in keep (converged, nonzero forcing) as a new column; the other
// problems (and problems whose force is already in the span) get zero columns. A solve of another
// precision than the stored columns' starts the space again.
void recycle_add(smob_ctx* c, const std::vector<double>& f, const double* const* parts, int nparts, int prec,
                 const std::vector<unsigned char>& keep) {
    if (std::none_of(keep.begin(), keep.end(), [](unsigned char k) { return k != 0; })) return;
    const size_t n = 3 * (size_t)c->M;
    const size_t n6 = 6 * (size_t)c->N;
    const int P = c->P;
    cudaStream_t st = c->st;
    if (!c->d_ru.p) {
        c->d_ru.alloc(sizeof(double) * n * kRecycleParts * kRecycleMax);
        c->d_rcoef.alloc(sizeof(double) * P * kRecycleMax);
        c->d_rscale.alloc(sizeof(double) * P);
        c->rq.assign(n6 * kRecycleMax, 0.0);
    }
    if (c->rk == kRecycleMax || prec != c->rprec) c->rk = 0;
    c->rprec = prec;
    const int k = c->rk;
    // host: q = F - Q coef (two classical Gram-Schmidt passes), per problem
    std::vector<double> q(n6, 0.0), coef((size_t)P * kRecycleMax, 0.0), fn2(P, 0.0), nu2(P, 0.0);
    for (int s = 0; s < c->N; ++s)
        if (keep[c->prob[s]])
            for (int i = 6 * s; i < 6 * s + 6; ++i) q[i] = f[i], fn2[c->prob[s]] += f[i] * f[i];
    for (int pass = 0; pass < 2 && k > 0; ++pass) {
        std::vector<double> d((size_t)P * kRecycleMax, 0.0);
        for (int s = 0; s < c->N; ++s)
            for (int i = 6 * s; i < 6 * s + 6; ++i)
                for (int j = 0; j < k; ++j) d[(size_t)c->prob[s] * kRecycleMax + j] += c->rq[n6 * j + i] * q[i];
        for (int s = 0; s < c->N; ++s)
            for (int i = 6 * s; i < 6 * s + 6; ++i)
                for (int j = 0; j < k; ++j) q[i] -= d[(size_t)c->prob[s] * kRecycleMax + j] * c->rq[n6 * j + i];
        for (size_t i = 0; i < d.size(); ++i) coef[i] += d[i];
    }
    for (int s = 0; s < c->N; ++s)
        for (int i = 6 * s; i < 6 * s + 6; ++i) nu2[c->prob[s]] += q[i] * q[i];
    std::vector<double> sc(P, 0.0);
    for (int p = 0; p < P; ++p) {
        const double nu = std::sqrt(nu2[p]);
        if (keep[p] && std::isfinite(nu) && nu > kRecycleDrop * std::sqrt(fn2[p])) sc[p] = 1.0 / nu;
    }
    for (int s = 0; s < c->N; ++s)
        for (int i = 6 * s; i < 6 * s + 6; ++i) c->rq[n6 * k + i] = q[i] * sc[c->prob[s]];
    // device: part_k = (v_k - U_k coef) / nu with the same coefficients
    KrylovLaunch L = c->kl();
    const unsigned char* act = c->d_active.as<unsigned char>();
    h2d(c, c->d_rcoef.p, coef.data(), sizeof(double) * coef.size());
    h2d(c, c->d_rscale.p, sc.data(), sizeof(double) * P);
    set_active(c, keep);
    for (int m = 0; m < kRecycleParts; ++m) {
        double* base = c->d_ru.as<double>() + n * m;
        double* u = base + n * kRecycleParts * k;
        CUDA_OK(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        if (m >= nparts || !parts[m]) continue;
        check_launch(c, launch_axpby_seg(L, 1.0, parts[m], 0.0, act, u, st));
        if (k > 0)
            check_launch(c, launch_update(L, base, (long long)(n * kRecycleParts), k, nullptr, c->d_rcoef.as<double>(),
                                          kRecycleMax, -1.0, act, u, st));
        check_launch(c, launch_scale(L, u, c->d_rscale.as<double>(), 1, false, act, u, st));
    }
    if (std::any_of(sc.begin(), sc.end(), [](double v) { return v != 0.0; })) c->rk++;
}

// ---------------------------------------------------------------- graph-driven restart loop
// The restart-cycle loop of solve_device as one CUDA graph whose control flow runs on the device:
//
//   decide                                     per problem: stop, or join the next cycle
//   while (a problem is in the cycle) {        conditional WHILE node
//     V_0 = r / beta, cycle init, step j = 0
//     while (a problem is active) {            conditional WHILE node
//       switch (j) { step(0) | ... | step(m-1) }   conditional SWITCH node: the Arnoldi step j
//       step control: j += 1, continue while a problem is active and j < m
//     }
//     x += V y; residual decision per problem
//     if (a problem takes the FP32 update) { r -= A32 dx }          conditional IF node
//     if (a problem takes the high-precision residual) { r = ... }  conditional IF node
//     beta = |r|; decide
//   }
//
// One graph launch per solve replaces the host loop's per-block synchronizations, per-cycle state
// round trips and the hundreds of launches of a solve. Every decision kernel applies the host loop's
// rules to the same values (krylov.cu), the bodies are the host loop's own launch sequences captured
// once per step index, and skipped bodies are exactly the steps the host loop does not launch or that
// launch kernels that return at once (every problem inactive), so both loops give the same bits.
struct LoopArgs {
    int m, maxit;
    bool mixed;
    int hp, cyc_prec;
    bool pc;
    double tol, inner_tol;
};

// captures the work f() issues on c->st (and on streams that join it) into graph g after the nodes
// deps; returns the nodes the capture ended on
template <typename F>
std::vector<cudaGraphNode_t> capture_into(smob_ctx* c, cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, F&& f) {
    CUDA_OK(cudaStreamBeginCaptureToGraph(c->st, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                          cudaStreamCaptureModeThreadLocal));
    std::vector<cudaGraphNode_t> tail;
    struct Capturing {
        smob_ctx* c;
        explicit Capturing(smob_ctx* x) : c(x) { c->capturing = true; }
        ~Capturing() { c->capturing = false; }
    } capturing(c);
    try {
        f();
        cudaStreamCaptureStatus status;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        CUDA_OK(cudaStreamGetCaptureInfo(c->st, &status, nullptr, nullptr, &d, nullptr, &nd));
        tail.assign(d, d + nd);
    } catch (...) {
        cudaGraph_t out = nullptr;
        cudaStreamEndCapture(c->st, &out);
        cudaGetLastError();
        throw;
    }
    cudaGraph_t out = nullptr;
    CUDA_OK(cudaStreamEndCapture(c->st, &out));
    return tail;
}

// a conditional node (while / switch / if) after deps; its body graphs in bodies[0 .. size-1]
cudaGraphNode_t add_conditional(cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h,
                                cudaGraphConditionalNodeType type, unsigned size, cudaGraph_t* bodies) {
    cudaGraphNodeParams prm = {};
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = h;
    prm.conditional.type = type;
    prm.conditional.size = size;
    cudaGraphNode_t node = nullptr;
    CUDA_OK(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &prm));
    for (unsigned i = 0; i < size; ++i) bodies[i] = prm.conditional.phGraph_out[i];
    return node;
}

// The launch sequences the graphs are built from (solve_device's own lambdas, so the host-driven
// path and the graphs issue the same kernels). The full-solve graph also takes the cold-start set-up
// and the final velocity.
struct SolveOps {
    std::function<void(int)> step;                    // Arnoldi step j on the active problems
    std::function<void(const double*)> upd;           // r -= A32 dx (active problems)
    std::function<void()> hp_residual;                // MIXED high-precision residual (active problems)
    std::function<void()> explicit_residual;          // r = b - A x in the solve's precision
    std::function<const double*()> cycle_update;      // x += V y (cycle problems); returns dx
    std::function<void()> pre;                        // cold start: rho, b, |b|, x = 0, r = b, |r|, track
    std::function<void()> post_from_hp, post_moved, post_mid, post_fresh, post_end;  // final velocity
};

// Appends the restart loop to graph G after deps (see the diagram above); returns its while node.
cudaGraphNode_t append_loop(smob_ctx* c, cudaGraph_t G, const std::vector<cudaGraphNode_t>& deps, const LoopArgs& a,
                            smob_ctx::LoopGraph& lg, const SolveOps& ops, bool first_decide) {
    const int P = c->P, m = a.m;
    cudaStream_t st = c->st;
    KrylovLaunch L = c->kl();
    auto* track = c->d_track.as<SolveTrack>();
    auto* sp = c->d_sparams.as<SolveParams>();
    unsigned char* act = c->d_active.as<unsigned char>();
    unsigned char* incyc = c->d_incycle.as<unsigned char>();
    unsigned char* updm = c->d_updmask.as<unsigned char>();
    unsigned char* hpm = c->d_hpmask.as<unsigned char>();
    KrylovState* ks = c->d_ks.as<KrylovState>();
    double* beta_d = c->d_beta.as<double>();
    double* norm = c->d_norm.as<double>();
    const double* r = c->d_r.as<double>();
    double* V = c->d_V.as<double>();
    int* jdev = c->d_jdev.as<int>();
    int* runs_j = c->d_runs_j.as<int>();
    auto count = [&](auto&& f) {
        const long long k0 = c->launches;
        f();
        return c->launches - k0;
    };
    cudaGraphConditionalHandle hc, hi, hsel, hu, hh;
    CUDA_OK(cudaGraphConditionalHandleCreate(&hc, G, 0, cudaGraphCondAssignDefault));
    std::vector<cudaGraphNode_t> tail = deps;
    if (first_decide)
        tail = capture_into(c, G, deps, [&] {
            lg.k_top += count([&] {
                check_launch(c, launch_loop_decide(P, false, track, ks, sp, nullptr, incyc, act, beta_d, a.maxit, hc,
                                                   st));
            });
        });
    cudaGraph_t body = nullptr;
    const cudaGraphNode_t wnode = add_conditional(G, tail, hc, cudaGraphCondTypeWhile, 1, &body);
    CUDA_OK(cudaGraphConditionalHandleCreate(&hi, body, 0, cudaGraphCondAssignDefault));
    CUDA_OK(cudaGraphConditionalHandleCreate(&hu, body, 0, cudaGraphCondAssignDefault));
    CUDA_OK(cudaGraphConditionalHandleCreate(&hh, body, 0, cudaGraphCondAssignDefault));
    long long kc = 0;
    tail = capture_into(c, body, {}, [&] {
        kc += count([&] {
            check_launch(c, launch_scale(L, r, beta_d, 1, true, act, V, st));
            check_launch(c, launch_cycle_init(L, m, incyc, beta_d, ks, c->d_H.as<double>(), c->d_g.as<double>(), st));
            check_launch(c, launch_inner_begin(jdev, hi, st));
        });
    });
    cudaGraph_t inner = nullptr;
    const cudaGraphNode_t inode = add_conditional(body, tail, hi, cudaGraphCondTypeWhile, 1, &inner);
    CUDA_OK(cudaGraphConditionalHandleCreate(&hsel, inner, 0, cudaGraphCondAssignDefault));
    std::vector<cudaGraph_t> steps(m, nullptr);
    const cudaGraphNode_t snode = add_conditional(inner, {}, hsel, cudaGraphCondTypeSwitch, m, steps.data());
    lg.k_step.assign(m, 0);
    for (int j = 0; j < m; ++j) capture_into(c, steps[j], {}, [&] { lg.k_step[j] = count([&] { ops.step(j); }); });
    long long knext = 0;
    capture_into(c, inner, {snode}, [&] {
        knext = count([&] { check_launch(c, launch_step_next(P, act, jdev, runs_j, m, hi, hsel, st)); });
    });
    for (long long& k : lg.k_step) k += knext;
    const double* dx = nullptr;
    tail = capture_into(c, body, {inode}, [&] {
        kc += count([&] {
            dx = ops.cycle_update();
            check_launch(c, launch_resid_decide(P, track, sp, incyc, updm, hpm, hu, hh, st));
        });
    });
    cudaGraph_t ub = nullptr, hb = nullptr;
    const cudaGraphNode_t unode = add_conditional(body, tail, hu, cudaGraphCondTypeIf, 1, &ub);
    capture_into(c, ub, {}, [&] {
        lg.k_upd = count([&] {
            CUDA_OK(cudaMemcpyAsync(act, updm, P, cudaMemcpyDeviceToDevice, st));
            ops.upd(dx);
            check_launch(c, launch_track_mark(P, track, updm, 0, st));
        });
    });
    const cudaGraphNode_t hnode = add_conditional(body, {unode}, hh, cudaGraphCondTypeIf, 1, &hb);
    capture_into(c, hb, {}, [&] {
        lg.k_hp = count([&] {
            CUDA_OK(cudaMemcpyAsync(act, hpm, P, cudaMemcpyDeviceToDevice, st));
            if (a.mixed) ops.hp_residual();
            else ops.explicit_residual();
            check_launch(c, launch_track_mark(P, track, hpm, 1, st));
        });
    });
    capture_into(c, body, {hnode}, [&] {
        kc += count([&] {
            CUDA_OK(cudaMemcpyAsync(act, incyc, P, cudaMemcpyDeviceToDevice, st));
            check_launch(c, launch_dots(L, r, 0, 1, r, act, norm, 1, 0, false, true, st));
            check_launch(c, launch_loop_decide(P, true, track, ks, sp, norm, incyc, act, beta_d, a.maxit, hc, st));
        });
    });
    lg.k_cycle = kc;
    return wnode;
}

// Appends the final velocity of the full-solve graph after deps: per problem u from u_hp (+ the FP32
// single layer of x - x_hp) or one high-precision single-layer pass, rho += x, rigid averages.
void append_final(smob_ctx* c, cudaGraph_t G, const std::vector<cudaGraphNode_t>& deps, smob_ctx::LoopGraph& lg,
                  const SolveOps& ops) {
    const int P = c->P;
    cudaStream_t st = c->st;
    auto* track = c->d_track.as<SolveTrack>();
    auto* sp = c->d_sparams.as<SolveParams>();
    unsigned char* act = c->d_active.as<unsigned char>();
    unsigned char* m_from = c->d_updmask.as<unsigned char>();
    unsigned char* m_moved = c->d_hpmask.as<unsigned char>();
    unsigned char* m_fresh = c->d_freshmask.as<unsigned char>();
    auto count = [&](auto&& f) {
        const long long k0 = c->launches;
        f();
        return c->launches - k0;
    };
    cudaGraphConditionalHandle hf, hm, hr;
    CUDA_OK(cudaGraphConditionalHandleCreate(&hf, G, 0, cudaGraphCondAssignDefault));
    CUDA_OK(cudaGraphConditionalHandleCreate(&hm, G, 0, cudaGraphCondAssignDefault));
    CUDA_OK(cudaGraphConditionalHandleCreate(&hr, G, 0, cudaGraphCondAssignDefault));
    auto tail = capture_into(c, G, deps, [&] {
        lg.k_post += count([&] {
            CUDA_OK(cudaMemsetAsync(c->d_u.p, 0, sizeof(double) * 3 * (size_t)c->M, st));
            check_launch(c, launch_final_decide(P, track, sp, m_from, m_moved, m_fresh, hf, hm, hr, st));
        });
    });
    cudaGraph_t bf = nullptr, bm = nullptr, br = nullptr;
    const cudaGraphNode_t nf = add_conditional(G, tail, hf, cudaGraphCondTypeIf, 1, &bf);
    capture_into(c, bf, {}, [&] {
        lg.k_from = count([&] {
            CUDA_OK(cudaMemcpyAsync(act, m_from, P, cudaMemcpyDeviceToDevice, st));
            ops.post_from_hp();
        });
    });
    const cudaGraphNode_t nm = add_conditional(G, {nf}, hm, cudaGraphCondTypeIf, 1, &bm);
    capture_into(c, bm, {}, [&] {
        lg.k_moved = count([&] {
            CUDA_OK(cudaMemcpyAsync(act, m_moved, P, cudaMemcpyDeviceToDevice, st));
            ops.post_moved();
        });
    });
    tail = capture_into(c, G, {nm}, [&] {
        lg.k_post += count([&] {
            CUDA_OK(cudaMemsetAsync(act, 1, P, st));
            ops.post_mid();
        });
    });
    const cudaGraphNode_t nr = add_conditional(G, tail, hr, cudaGraphCondTypeIf, 1, &br);
    capture_into(c, br, {}, [&] {
        lg.k_fresh = count([&] {
            CUDA_OK(cudaMemcpyAsync(act, m_fresh, P, cudaMemcpyDeviceToDevice, st));
            ops.post_fresh();
        });
    });
    capture_into(c, G, {nr}, [&] {
        lg.k_post += count([&] {
            CUDA_OK(cudaMemsetAsync(act, 1, P, st));
            ops.post_end();
        });
    });
}

// Runs the restart loop (full = false: the per-problem state goes in and comes back in one copy each
// way) or the whole cold-start solve (full = true: set-up, loop and final velocity; the state only
// comes back) as one graph launch, built on first use per LoopArgs shape. Returns false, with nothing
// changed, when the graph cannot be built (conditional nodes unavailable): the caller runs the host
// path instead.
bool run_loop_graph(smob_ctx* c, const LoopArgs& a, const SolveOps& ops, bool full, std::vector<char>& done,
                    std::vector<char>& conv, std::vector<double>& beta, std::vector<double>& bnorm,
                    std::vector<char>& hp_now, std::vector<char>& hp_resid_done, std::vector<char>& x_moved,
                    std::vector<int>& cycles, std::vector<int>& passes64, std::vector<int>& passes32x) {
    const int P = c->P, m = a.m;
    cudaStream_t st = c->st;
    auto* track = c->d_track.as<SolveTrack>();
    auto* sp = c->d_sparams.as<SolveParams>();
    int* runs_j = c->d_runs_j.as<int>();
    const std::vector<int> key{full ? 1 : 0, a.mixed ? 1 : 0, a.hp, a.cyc_prec, a.pc ? 1 : 0, m, a.maxit};
    auto it = c->loop_graphs.find(key);
    if (it == c->loop_graphs.end()) {
        smob_ctx::LoopGraph lg;
        const long long before = c->launches;
        cudaGraph_t G = nullptr;
        try {
            CUDA_OK(cudaGraphCreate(&G, 0));
            std::vector<cudaGraphNode_t> tail;
            if (full)
                tail = capture_into(c, G, {}, [&] {
                    const long long k0 = c->launches;
                    ops.pre();
                    lg.k_top += c->launches - k0;
                });
            const cudaGraphNode_t wnode = append_loop(c, G, tail, a, lg, ops, true);
            if (full) append_final(c, G, {wnode}, lg, ops);
            // each kernel node keeps the priority of the stream it was captured on (main above far field)
            CUDA_OK(cudaGraphInstantiate(&lg.exec, G, cudaGraphInstantiateFlagUseNodePriority));
            cudaGraphDestroy(G);
            c->launches = before;
        } catch (const SmobError&) {
            if (G) cudaGraphDestroy(G);
            cudaGetLastError();
            c->launches = before;
            c->loop_graph_ok = false;
            return false;
        }
        it = c->loop_graphs.emplace(key, std::move(lg)).first;
    }
    const smob_ctx::LoopGraph& lg = it->second;
    if (!full) {
        std::vector<SolveTrack> tr(P);
        for (int p = 0; p < P; ++p)
            tr[p] = SolveTrack{bnorm[p], beta[p], done[p], conv[p], hp_now[p], hp_resid_done[p], x_moved[p],
                               cycles[p], passes64[p], passes32x[p]};
        h2d(c, track, tr.data(), sizeof(SolveTrack) * P);
    }
    SolveParams prm{};
    prm.tol = a.tol;
    prm.inner_tol = a.inner_tol;
    prm.mixed = a.mixed ? 1 : 0;
    prm.max_cycles = a.maxit + 1;
    h2d(c, sp, &prm, sizeof(prm));
    CUDA_OK(cudaMemsetAsync(runs_j, 0, sizeof(int) * m, st));
    CUDA_OK(cudaGraphLaunch(lg.exec, st));
    auto* tr_s = static_cast<SolveTrack*>(stage_alloc(c, sizeof(SolveTrack) * P));
    auto* sp_s = static_cast<SolveParams*>(stage_alloc(c, sizeof(SolveParams)));
    auto* rj_s = static_cast<int*>(stage_alloc(c, sizeof(int) * m));
    CUDA_OK(cudaMemcpyAsync(tr_s, track, sizeof(SolveTrack) * P, cudaMemcpyDeviceToHost, st));
    CUDA_OK(cudaMemcpyAsync(sp_s, sp, sizeof(SolveParams), cudaMemcpyDeviceToHost, st));
    CUDA_OK(cudaMemcpyAsync(rj_s, runs_j, sizeof(int) * m, cudaMemcpyDeviceToHost, st));
    stage_sync(c);
    if (sp_s->overrun) {
        c->loop_graph_ok = false;
        throw SmobError(SMOB_ERR_STATE, "the graph-driven restart loop ran more cycles than iterations (results void)");
    }
    for (int p = 0; p < P; ++p) {
        const SolveTrack& t = tr_s[p];
        bnorm[p] = t.bnorm;
        beta[p] = t.beta;
        done[p] = char(t.done);
        conv[p] = char(t.conv);
        hp_now[p] = char(t.hp_now);
        hp_resid_done[p] = char(t.hp_done);
        x_moved[p] = char(t.x_moved);
        cycles[p] = t.cycles;
        passes64[p] = t.passes64;
        passes32x[p] = t.passes32x;
    }
    long long k = lg.k_top + (long long)sp_s->cycles_run * lg.k_cycle + (long long)sp_s->upd_run * lg.k_upd +
                  (long long)sp_s->hp_run * lg.k_hp + lg.k_post + (long long)sp_s->fin_from * lg.k_from +
                  (long long)sp_s->fin_moved * lg.k_moved + (long long)sp_s->fin_fresh * lg.k_fresh;
    for (int j = 0; j < m; ++j) k += (long long)rj_s[j] * lg.k_step[j];
    c->launches += k;
    c->host_calls += 1;
    return true;
}

// New far-field tolerances: both coarse sets rebuilt (the FP32 one and the float-float one).
void rebuild_far_sets(smob_ctx* c, double eps, double eps_hp) {
    AllocStreamScope as(c->st);
    c->drop_graphs();  // captured blocks hold the old coarse tables
    for (auto& kv : c->multi) smob_destroy(kv.second);  // several-RHS copies follow the new tolerance
    c->multi.clear();
    c->c32.eps = eps > 0 ? eps : 0.0;
    c->chp.eps = eps_hp > 0 ? eps_hp : 0.0;
    c->rk = 0;  // recycled residuals belong to the old operators
    build_coarse(c);
    bind_geom(c);
    coarse_grids(c);
    CUDA_OK(cudaStreamSynchronize(c->st));
}

// The float-float set's tolerance follows the solves (unless the caller set it): one decade below the
// tolerance a solve asks for, at most kCoarseEpsHpDefault (its value at creation), at least 1e-12. A
// solve asking for more than the set gives tightens it once (both sets rebuilt); it is never loosened.
void fit_eps_hp(smob_ctx* c, double tol) {
    if (!c->eps_hp_auto || c->chp.eps <= 0) return;
    const double want = std::min(kCoarseEpsHpDefault, std::max(0.1 * tol, 1e-12));
    if (want < c->chp.eps) rebuild_far_sets(c, c->c32.eps, want);
}

// the mobility solve on device pointers (SphereSTKMobMat::solveMob, BIE/SphereSTKMobMat.cpp:146-286)
smob_status solve_device(smob_ctx* c, const double* d_force, double* d_vel, double* d_density,
                         const smob_solve_opts* o, smob_problem_stats* stats) {
    const int m = std::max(1, o->restart);
    const bool mixed = o->precision == SMOB_PREC_MIXED;
    const double tol = o->tol;
    const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-5;
    const int maxit = std::max(1, o->max_iters);
    // high-precision operator (b, refinement residuals, final velocity) and the cycle operator;
    // SMOB_PREC_FLOAT_FLOAT runs the plain restarted GMRES with the float-float far field throughout
    const bool ffar = o->precision == SMOB_PREC_FLOAT_FLOAT;
    const int hp = (mixed || ffar) ? OP_DF : OP_FP64;
    const int cyc_prec = mixed ? OP_FP32 : hp;
    if (hp == OP_DF) fit_eps_hp(c, tol);  // before anything is captured: it rebuilds the coarse sets
    ensure_tuned(c);  // before any capture: the tuner synchronizes
    ensure_solver(c, m);
    const size_t n = 3 * (size_t)c->M;
    const int P = c->P;
    KrylovLaunch L = c->kl();
    cudaStream_t st = c->st;
    double* V = c->d_V.as<double>();
    double* w = c->d_w.as<double>();
    double* r = c->d_r.as<double>();
    double* x = c->d_x.as<double>();
    double* b = c->d_b.as<double>();
    double* rho = c->d_rho.as<double>();
    double* u = c->d_u.as<double>();
    unsigned char* act = c->d_active.as<unsigned char>();
    unsigned char* incyc = c->d_incycle.as<unsigned char>();
    KrylovState* ks = c->d_ks.as<KrylovState>();
    // Optional right preconditioner P: per sphere the exact inverse of its own I/2 + K_PV + L
    // (block diagonal, one sphere-kernel pass in the cycle precision). GMRES then builds its
    // Krylov space for A P while every residual stays that of A x = b.
    const bool pc = o->precond != 0;
    double* pz = nullptr;
    if (pc) {
        c->d_pz.alloc(sizeof(double) * n);
        pz = c->d_pz.as<double>();
    }
    auto apply_precond = [&](const double* in, double* out) {
        CUDA_OK(cudaMemsetAsync(out, 0, sizeof(double) * n, st));
        check_launch(c, launch_sphere_op(c->g, in, out, 2.0, 1.0, 4, 0.0, nullptr, cyc_prec == OP_FP32, st));
    };

    std::vector<unsigned char> all(P, 1);
    std::vector<int> passes64(P, 0), cycles(P, 0), passes32x(P, 0);
    std::vector<char> hp_resid_done(P, 0);  // a high-precision residual after a cycle exists
    // MIXED: beta[p] is a high-precision residual norm (or one updated from it by a small FP32 step);
    // only such a residual may end a problem's solve
    std::vector<char> hp_now(P, mixed ? 0 : 1);
    std::vector<char> x_moved(P, 0);  // MIXED: x changed since the last high-precision residual
    double *dens = nullptr, *uhp = nullptr, *xhp = nullptr;
    if (mixed) {
        c->d_dens.alloc(sizeof(double) * n);
        c->d_uhp.alloc(sizeof(double) * n);
        c->d_xhp.alloc(sizeof(double) * n);
        c->d_partial64_sl.alloc(sizeof(double) * c->partial64);  // op_apply_hp_both (before any capture)
        dens = c->d_dens.as<double>();
        uhp = c->d_uhp.as<double>();
        xhp = c->d_xhp.as<double>();
    }
    // MIXED: one fused high-precision pass on the problems in mask gives r = -(I/2 + K)(rho + x) - L x
    // and the single layer u_hp = S[rho + x] (the final velocity then needs only S32[x - x_hp])
    // the device work of hp_residual on the problems already marked active
    auto hp_residual_ops = [&]() {
        CUDA_OK(cudaMemcpyAsync(dens, rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        check_launch(c, launch_axpby_seg(L, 1.0, x, 1.0, act, dens, st));
        CUDA_OK(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
        op_apply_hp_both(c, dens, u, -0.5, -1.0, w, 1.0);
        op_apply(c, x, u, 0.0, 0.0, 0.0, -1.0, OP_FP64);  // - L x (per-sphere rigid modes)
        check_launch(c, launch_axpby_seg(L, 1.0, u, 0.0, act, r, st));
        check_launch(c, launch_axpby_seg(L, 1.0, w, 0.0, act, uhp, st));
        check_launch(c, launch_axpby_seg(L, 1.0, x, 0.0, act, xhp, st));
    };
    auto hp_residual = [&](const std::vector<unsigned char>& mask) {
        set_active(c, mask);
        hp_residual_ops();
        for (int p = 0; p < P; ++p)
            if (mask[p]) passes64[p]++, hp_resid_done[p] = 1, hp_now[p] = 1, x_moved[p] = 0;
    };
    const long long hs = (long long)m * (m + 1);
    // one Arnoldi step: w = A V_j (A = I/2 + K + L, SphereSTKMobMat.cpp:17), CGS2 into H[:, j],
    // Givens update and the per-problem stop test on the device (problems that stop skip all
    // later work through the active flags)
    auto step = [&](int j) {
        const double* Vj = V + n * j;
        if (pc) {  // right preconditioning: w = A P V_j
            apply_precond(Vj, pz);
            Vj = pz;
        }
        CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
        op_apply(c, Vj, w, 0.5, 0.0, 1.0, 1.0, cyc_prec);
        double* Hcol = c->d_H.as<double>() + (long long)j * (m + 1);
        double* hscr = c->d_y.as<double>();
        for (int pass = 0; pass < 2; ++pass) {
            check_launch(c, launch_dots(L, V, (long long)n, j + 1, w, act, hscr, m, 0, false, false, st, Hcol, hs,
                                        pass == 1));
            if (pass == 0) check_launch(c, launch_update(L, V, (long long)n, j + 1, nullptr, hscr, m, -1.0, act, w, st));
        }
        // second update, |w| and the Givens step in one kernel
        check_launch(c, launch_update_norm_givens(L, V, (long long)n, j + 1, hscr, m, act, w, c->d_hn.as<double>(), j, m,
                                                  ks, c->d_H.as<double>(), c->d_g.as<double>(),
                                                  c->d_cs.as<double>(), c->d_sn.as<double>(), maxit, st));
        if (j + 1 < m) check_launch(c, launch_scale(L, w, c->d_hn.as<double>(), 1, true, act, V + n * (j + 1), st));
    };
    // residual of the FP32-update problems (MIXED): r -= A32 dx on the problems already marked active
    auto upd_ops = [&](const double* dx) {
        CUDA_OK(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        op_apply(c, dx, u, 0.5, 0.0, 1.0, 1.0, OP_FP32);
        check_launch(c, launch_axpby_seg(L, -1.0, u, 1.0, act, r, st));
    };
    // explicit residual r = b - A x in the solve's precision (FP64 / float-float solves)
    auto explicit_residual_ops = [&]() {
        CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
        op_apply(c, x, w, 0.5, 0.0, 1.0, 1.0, hp);
        check_launch(c, launch_axpby_seg(L, 1.0, b, 0.0, act, r, st));
        check_launch(c, launch_axpby_seg(L, -1.0, w, 1.0, act, r, st));
    };
    // x += V y (P V y when preconditioned) for the problems of the cycle (after the Arnoldi steps);
    // returns the correction dx
    auto cycle_update_ops = [&]() -> const double* {
        check_launch(c, launch_trisolve(L, m, incyc, ks, c->d_H.as<double>(), c->d_g.as<double>(), c->d_y.as<double>(),
                                        c->d_kc.as<int>(), st));
        CUDA_OK(cudaMemcpyAsync(act, incyc, P, cudaMemcpyDeviceToDevice, st));
        CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
        check_launch(c, launch_update(L, V, (long long)n, m, c->d_kc.as<int>(), c->d_y.as<double>(), m, 1.0, act, w, st));
        double* dx = w;  // the correction of this cycle: V y, or P V y when preconditioned
        if (pc) {
            apply_precond(w, pz);
            dx = pz;
        }
        check_launch(c, launch_axpby_seg(L, 1.0, dx, 1.0, act, x, st));
        return dx;
    };

    // step 4's pieces (final velocity), on the problems already marked active
    auto post_from_hp = [&]() { check_launch(c, launch_axpby_seg(L, 1.0, uhp, 0.0, act, u, st)); };
    auto post_moved = [&]() {
        check_launch(c, launch_axpby_seg(L, 1.0, x, 0.0, act, w, st));
        check_launch(c, launch_axpby_seg(L, -1.0, xhp, 1.0, act, w, st));
        op_apply(c, w, u, 0.0, 1.0, 0.0, 0.0, OP_FP32);
    };
    auto post_mid = [&]() { check_launch(c, launch_axpby_seg(L, 1.0, x, 1.0, act, rho, st)); };
    auto post_fresh = [&]() { op_apply(c, rho, u, 0.0, 1.0, 0.0, 0.0, hp); };
    auto post_end = [&](double* vel) {
        check_launch(c, launch_rigid_average(c->g, u, 1.0 / c->viscosity, vel, st));
        CUDA_OK(cudaMemcpyAsync(c->d_xlast.p, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    };
    // step 1: rigid density; step 2: b = -(I/2 + K) rho. FP64 / float-float: in the solve's precision.
    // MIXED: with the FP32 operator. b only seeds the first inner cycle and scales the tolerance; every
    // high-precision residual is formed directly as r = -(I/2 + K)(rho + x) - L x, so b's FP32 error
    // never reaches a residual that decides convergence.
    auto pre_b = [&](const double* force) {
        check_launch(c, launch_rigid_density(c->g, force, rho, st));
        CUDA_OK(cudaMemsetAsync(b, 0, sizeof(double) * n, st));
        op_apply(c, rho, b, -0.5, 0.0, -1.0, 0.0, mixed ? OP_FP32 : hp);
    };

    SolveOps ops;
    ops.step = step;
    ops.upd = upd_ops;
    ops.hp_residual = hp_residual_ops;
    ops.explicit_residual = explicit_residual_ops;
    ops.cycle_update = cycle_update_ops;
    // the cold start of the full-solve graph: steps 1-2, x = 0, r = b and the per-problem state
    ops.pre = [&]() {
        CUDA_OK(cudaMemsetAsync(act, 1, P, st));
        CUDA_OK(cudaMemsetAsync(ks, 0, sizeof(KrylovState) * P, st));
        pre_b(c->d_force.as<double>());
        check_launch(c, launch_dots(L, b, 0, 1, b, act, c->d_bnorm.as<double>(), 1, 0, false, true, st));
        CUDA_OK(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
        CUDA_OK(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        check_launch(c, launch_dots(L, r, 0, 1, r, act, c->d_norm.as<double>(), 1, 0, false, true, st));
        check_launch(c, launch_track_init(P, mixed, c->d_bnorm.as<double>(), c->d_norm.as<double>(),
                                          c->d_track.as<SolveTrack>(), st));
    };
    ops.post_from_hp = post_from_hp;
    ops.post_moved = post_moved;
    ops.post_mid = post_mid;
    ops.post_fresh = post_fresh;
    ops.post_end = [&]() { post_end(c->d_vel.as<double>()); };

    const bool graph_path = c->use_graphs && c->loop_graph_on && c->loop_graph_ok && !c->prof;
    const LoopArgs la{m, maxit, mixed, hp, cyc_prec, pc, tol, inner_tol};
    std::vector<double> bnorm(P, 0.0), beta(P, 0.0);
    std::vector<char> done(P, 0), conv(P, 0);
    std::vector<KrylovState> kst(P);
    bool nonfinite_any = false;
    // A cold-start solve is one graph launch (set-up, restart loop, final velocity); the caller's
    // force and velocity buffers are copied to and from the context's own, which the graph holds.
    bool full_done = false;
    if (graph_path && o->warm_start == SMOB_WARM_NONE) {
        if (d_force != c->d_force.as<double>())
            CUDA_OK(cudaMemcpyAsync(c->d_force.p, d_force, sizeof(double) * 6 * c->N, cudaMemcpyDeviceToDevice, st));
        full_done = run_loop_graph(c, la, ops, true, done, conv, beta, bnorm, hp_now, hp_resid_done, x_moved, cycles,
                                   passes64, passes32x);
        if (full_done) {
            if (d_vel != c->d_vel.as<double>())
                CUDA_OK(cudaMemcpyAsync(d_vel, c->d_vel.p, sizeof(double) * 6 * c->N, cudaMemcpyDeviceToDevice, st));
            if (d_density) CUDA_OK(cudaMemcpyAsync(d_density, rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            c->have_xlast = true;
        }
    }
    const bool recycle = o->warm_start == 2;
    if (!full_done) {
        set_active(c, all);
        std::vector<KrylovState> hks(P);
        for (auto& k : hks) k = KrylovState{0, 0, 0, 0, 0, 0, 0};
        h2d(c, ks, hks.data(), sizeof(KrylovState) * P);

        pre_b(d_force);
        for (int p = 0; p < P; ++p) (mixed ? passes32x[p] : passes64[p])++;
        bnorm = seg_norms(c, b, act);

        // initial guess (SphereSTKMobMat.cpp:222): warm start from the previous solution, zero, or
        // (warm_start 2) the combination of recycled earlier solutions closest to this b
        std::vector<double> hforce;
        if (recycle) {
            hforce.resize(6 * (size_t)c->N);
            d2h(c, hforce.data(), d_force, sizeof(double) * hforce.size());
        }
        if (recycle && c->rk > 0) {
            // MIXED from MIXED columns: a force in the span (to far below the tolerance) takes the
            // combined residual, u_hp and x_hp as well, which are those of the combined solution (every
            // part is linear in the force): no operator pass is needed to know where it stands
            const bool state = mixed && c->rprec == SMOB_PREC_MIXED;
            double* parts[kRecycleParts] = {x, state ? r : nullptr, state ? uhp : nullptr, state ? xhp : nullptr};
            const std::vector<double> est = recycle_guess(c, hforce, parts, kRecycleParts);
            std::vector<unsigned char> good(P, 0), poor(P, 0);
            bool any_good = false, any_poor = false;
            for (int p = 0; p < P; ++p) {
                if (state && est[p] <= 1e-2 * tol) hp_resid_done[p] = 1, hp_now[p] = 1, x_moved[p] = 1;
                else if (mixed && est[p] <= kRecycleHpFirst) good[p] = 1, any_good = true;
                else poor[p] = 1, any_poor = true;
            }
            if (any_poor) {
                set_active(c, poor);
                CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
                op_apply(c, x, w, 0.5, 0.0, 1.0, 1.0, mixed ? OP_FP32 : hp);
                check_launch(c, launch_axpby_seg(L, 1.0, b, 0.0, act, r, st));
                check_launch(c, launch_axpby_seg(L, -1.0, w, 1.0, act, r, st));
                for (int p = 0; p < P; ++p)
                    if (poor[p]) (mixed ? passes32x[p] : passes64[p])++, x_moved[p] = mixed ? 1 : 0;
            }
            if (any_good) hp_residual(good);
            set_active(c, all);
        } else if (o->warm_start && c->have_xlast) {
            CUDA_OK(cudaMemcpyAsync(x, c->d_xlast.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            CUDA_OK(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
            op_apply(c, x, w, 0.5, 0.0, 1.0, 1.0, mixed ? OP_FP32 : hp);
            for (int p = 0; p < P; ++p) (mixed ? passes32x[p] : passes64[p])++;
            if (mixed) std::fill(x_moved.begin(), x_moved.end(), 1);
            check_launch(c, launch_axpby_seg(L, 1.0, b, 0.0, act, r, st));
            check_launch(c, launch_axpby_seg(L, -1.0, w, 1.0, act, r, st));
        } else {
            CUDA_OK(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
            CUDA_OK(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        }
        beta = seg_norms(c, r, act);
        for (int p = 0; p < P; ++p) {
            if (!std::isfinite(bnorm[p]) || !std::isfinite(beta[p])) {
                done[p] = 1;
                nonfinite_any = true;
            } else if (bnorm[p] < 1e-5) {  // forcing is zero: density correction is zero (SphereSTKMobMat.cpp:217)
                done[p] = 1;
                conv[p] = 1;
            }
        }
        if (std::any_of(done.begin(), done.end(), [](char d) { return d; })) {
            // zero the correction of finished problems
            std::vector<unsigned char> zm(P, 0);
            for (int p = 0; p < P; ++p) zm[p] = done[p] ? 1 : 0;
            set_active(c, zm);
            check_launch(c, launch_axpby_seg(L, 0.0, x, 0.0, act, x, st));
        }

        // Restart cycles in lockstep over the problems still running. FP64: each cycle is a
        // GMRES(m) cycle on the FP64 operator, followed by the explicit residual (Belos' restart).
        // MIXED: each cycle solves A d = r with the FP32 operator (FP64 Arnoldi/Givens) to a relative
        // inner tolerance, x += d, and the refinement residual r = b - A x uses the FP64 operator.
        std::vector<unsigned char> hact(P);
        bool loop_done = false;
        if (graph_path)
            loop_done = run_loop_graph(c, la, ops, false, done, conv, beta, bnorm, hp_now, hp_resid_done, x_moved, cycles,
                                       passes64, passes32x);
        while (!loop_done) {
            d2h(c, kst.data(), ks, sizeof(KrylovState) * P);
            std::vector<unsigned char> cyc(P, 0);
            int ncyc = 0;
            for (int p = 0; p < P; ++p) {
                if (done[p]) continue;
                if (beta[p] / bnorm[p] < tol && hp_now[p]) {
                    done[p] = 1;
                    conv[p] = 1;
                    continue;
                }
                if (kst[p].iters >= maxit || kst[p].nonfinite) {
                    done[p] = 1;
                    continue;
                }
                cyc[p] = 1;
                ++ncyc;
                cycles[p]++;
                kst[p].tol_abs = mixed ? std::max(inner_tol * beta[p], 0.5 * tol * bnorm[p]) : tol * bnorm[p];
                kst[p].cycle_fp32 = mixed ? 1 : 0;
            }
            if (ncyc == 0) break;
            h2d(c, ks, kst.data(), sizeof(KrylovState) * P);
            h2d(c, incyc, cyc.data(), P);
            h2d(c, c->d_beta.p, beta.data(), sizeof(double) * P);
            set_active(c, cyc);
            check_launch(c, launch_scale(L, r, c->d_beta.as<double>(), 1, true, act, V, st));
            check_launch(c, launch_cycle_init(L, m, incyc, c->d_beta.as<double>(), ks, c->d_H.as<double>(),
                                              c->d_g.as<double>(), st));
            // Steps run in blocks of kGraphBlock; with graphs on, each block is captured once per context
            // (per block start, cycle precision and restart length) and replayed, and the host looks at
            // the active flags only between blocks (steps after every problem stopped inside a block
            // launch kernels that return at once). A profiled solve checks after every step, so each
            // kernel it times did its full work.
            const bool graphs = c->use_graphs && !c->prof;
            const int blk = c->prof ? 1 : kGraphBlock;
            for (int j0 = 0; j0 < m; j0 += blk) {
                const int cnt = std::min(blk, m - j0);
                if (graphs) {
                    const long long key = (((long long)cyc_prec * 2 + (pc ? 1 : 0)) * 4096 + m) * 4096 + j0;
                    auto it = c->graphs.find(key);
                    if (it == c->graphs.end()) {
                        const long long before = c->launches;
                        cudaGraph_t gr;
                        CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                        c->capturing = true;
                        try {
                            for (int j = j0; j < j0 + cnt; ++j) step(j);
                        } catch (...) {
                            c->capturing = false;
                            cudaGraph_t t = nullptr;
                            cudaStreamEndCapture(st, &t);
                            if (t) cudaGraphDestroy(t);
                            cudaGetLastError();
                            c->launches = before;
                            throw;
                        }
                        c->capturing = false;
                        CUDA_OK(cudaStreamEndCapture(st, &gr));
                        cudaGraphExec_t ex;
                        CUDA_OK(cudaGraphInstantiate(&ex, gr, cudaGraphInstantiateFlagUseNodePriority));
                        cudaGraphDestroy(gr);
                        it = c->graphs.emplace(key, smob_ctx::Graph{ex, c->launches - before}).first;
                        c->launches = before;
                    }
                    CUDA_OK(cudaGraphLaunch(it->second.exec, st));
                    c->launches += it->second.kernels;
                    c->host_calls += 1;
                } else {
                    for (int j = j0; j < j0 + cnt; ++j) step(j);
                }
                d2h(c, hact.data(), act, P);
                if (std::none_of(hact.begin(), hact.end(), [](unsigned char a) { return a != 0; })) break;
            }
            // d = V y and x += d for the problems of this cycle
            const double* dx = cycle_update_ops();
            // Residual, decided per problem (so a problem takes the same steps alone or in any batch).
            // FP64 / float-float solves: explicit r = b - A x with the cycle's operator (Belos' restart).
            // MIXED, once the previous high-precision residual is below 1e-4 |b|: r <- r - A32 d, whose
            // FP32 error ~eps32 * kappa * |r_prev| (<= ~1e-10 |b|) is far below the 1e-8 target.
            // MIXED otherwise: one fused high-precision pass gives r = -(I/2 + K)(rho + x) - L x and the
            // single layer u_hp = S[rho + x] (the final velocity then needs only S32[x - x_hp]).
            std::vector<unsigned char> upd(P, 0), hpres(P, 0);
            bool any_upd = false, any_hp = false;
            for (int p = 0; p < P; ++p) {
                if (!cyc[p]) continue;
                if (mixed && hp_resid_done[p] && beta[p] <= 1e-4 * bnorm[p]) upd[p] = 1, any_upd = true;
                else hpres[p] = 1, any_hp = true;
            }
            if (any_upd) {
                set_active(c, upd);
                upd_ops(dx);
                for (int p = 0; p < P; ++p)
                    if (upd[p]) passes32x[p]++, x_moved[p] = 1;
            }
            if (any_hp && mixed) {
                hp_residual(hpres);
            } else if (any_hp) {
                set_active(c, hpres);
                explicit_residual_ops();
                for (int p = 0; p < P; ++p)
                    if (hpres[p]) passes64[p]++, hp_resid_done[p] = 1, hp_now[p] = 1, x_moved[p] = 0;
            }
            set_active(c, cyc);
            std::vector<double> nb = seg_norms(c, r, act);
            for (int p = 0; p < P; ++p)
                if (cyc[p]) beta[p] = nb[p];
        }

        // step 4: rho += mu; u = S[rho] (high precision); rigid averages / viscosity (SphereSTKMobMat.cpp:243-285).
        // MIXED problems with a high-precision residual already hold u_hp = S[rho + x_hp]:
        // u = u_hp + S32[x - x_hp], the FP32 part acting on the last small correction only.
        CUDA_OK(cudaMemsetAsync(u, 0, sizeof(double) * n, st));
        std::vector<unsigned char> from_hp(P, 0), moved(P, 0), fresh(P, 0);
        bool any_from_hp = false, any_moved = false, any_fresh = false;
        for (int p = 0; p < P; ++p) {
            if (mixed && hp_resid_done[p]) {
                from_hp[p] = 1, any_from_hp = true;
                if (x_moved[p]) moved[p] = 1, any_moved = true;
            } else {
                fresh[p] = 1, any_fresh = true;
            }
        }
        if (any_from_hp) {
            set_active(c, from_hp);
            post_from_hp();
        }
        if (any_moved) {
            set_active(c, moved);
            post_moved();
            for (int p = 0; p < P; ++p)
                if (moved[p]) passes32x[p]++;
        }
        set_active(c, all);
        post_mid();
        if (any_fresh) {
            set_active(c, fresh);
            post_fresh();
            for (int p = 0; p < P; ++p)
                if (fresh[p]) passes64[p]++;
            set_active(c, all);
        }
        post_end(d_vel);
        if (d_density) CUDA_OK(cudaMemcpyAsync(d_density, rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        c->have_xlast = true;
        if (recycle) {
            std::vector<unsigned char> keep(P, 0);
            for (int p = 0; p < P; ++p) keep[p] = conv[p] && std::isfinite(bnorm[p]) && bnorm[p] >= 1e-5 ? 1 : 0;
            const double* parts[kRecycleParts] = {x, mixed ? r : nullptr, uhp, xhp};
            recycle_add(c, hforce, parts, kRecycleParts, o->precision, keep);
            set_active(c, all);
        }
    }  // regular path
    auto* kst_s = static_cast<KrylovState*>(stage_alloc(c, sizeof(KrylovState) * P));
    auto* err_s = static_cast<int*>(stage_alloc(c, sizeof(int)));
    CUDA_OK(cudaMemcpyAsync(kst_s, ks, sizeof(KrylovState) * P, cudaMemcpyDeviceToHost, st));
    CUDA_OK(cudaMemcpyAsync(err_s, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    stage_sync(c);
    std::copy(kst_s, kst_s + P, kst.begin());
    const int dev_err = *err_s;
    if (dev_err != 0) {
        CUDA_OK(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), st));
        throw SmobError(SMOB_ERR_CUDA, "a tensor-core near-field kernel gave up waiting for its MMAs (results void)");
    }

    smob_status worst = SMOB_OK;
    for (int p = 0; p < P; ++p) {
        smob_status sp = SMOB_OK;
        if (!std::isfinite(bnorm[p]) || kst[p].nonfinite || !std::isfinite(beta[p])) sp = SMOB_ERR_NONFINITE;
        else if (!conv[p]) sp = SMOB_ERR_NOT_CONVERGED;
        if (sp != SMOB_OK && worst == SMOB_OK) worst = sp;
        if (stats) {
            smob_problem_stats& s = stats[p];
            s.status = sp;
            s.iterations = kst[p].iters;
            s.refinements = cycles[p];
            s.operator_passes_fp64 = passes64[p] + kst[p].passes64;
            s.operator_passes_fp32 = kst[p].passes32 + passes32x[p];
            s.bnorm = bnorm[p];
            s.relres = bnorm[p] < 1e-5 ? 0.0 : beta[p] / bnorm[p];
        }
    }
    if (nonfinite_any && worst == SMOB_OK) worst = SMOB_ERR_NONFINITE;
    if (worst == SMOB_ERR_NONFINITE) g_err = "non-finite values in the mobility solve";
    else if (worst == SMOB_ERR_NOT_CONVERGED) g_err = "GMRES stopped at its iteration limit";
    return worst;
}

// Reads and clears the device error word (DevGeom::err) after the stream's work so far; a kernel
// that gave up a bounded wait (tensor-core near field) wrote nothing, so the call's results are void.
void check_device_error(smob_ctx* c) {
    int h = 0;
    d2h(c, &h, c->d_err.p, sizeof(int));
    if (h != 0) {
        CUDA_OK(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->st));
        throw SmobError(SMOB_ERR_CUDA, "a tensor-core near-field kernel gave up waiting for its MMAs (results void)");
    }
}

template <typename F>
smob_status guarded(F&& f) {
    try {
        return f();
    } catch (const SmobError& e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_err = "host allocation failed";
        return SMOB_ERR_NOMEM;
    } catch (const std::exception& e) {
        g_err = e.what();
        return SMOB_ERR_CUDA;
    }
}

void need(bool cond, const char* msg) {
    if (!cond) throw SmobError(SMOB_ERR_ARG, msg);
}

void set_device(const smob_ctx* c) { CUDA_OK(cudaSetDevice(c->device)); }

// Entry-point scope: the context's device, and its main stream for every device buffer the call
// allocates or frees, so a lazily allocated buffer is ordered with the context's own work instead of
// the legacy default stream that all threads share.
struct CtxScope {
    AllocStreamScope alloc;
    explicit CtxScope(const smob_ctx* c) : alloc((set_device(c), c->st)) {}
};

// the context's main and side streams (non-blocking, priorities prio and far_prio: 0 is the default)
// and the fork/join events of the operator passes
// cuGreenCtxStreamCreate, reached through the runtime (the library does not link libcuda)
using GreenStreamFn = int (*)(void** stream, void* green_ctx, unsigned flags, int priority);
GreenStreamFn green_stream_fn() {
    static GreenStreamFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuGreenCtxStreamCreate", &f, 12050, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<GreenStreamFn>(f);
    }();
    return fn;
}

// green: a green context (an SM partition of the device, CUgreenCtx) whose streams the context runs on,
// or null for ordinary streams (the whole device)
void create_streams(smob_ctx* c, int prio, int far_prio, void* green = nullptr) {
    if (green) {
        GreenStreamFn fn = green_stream_fn();
        if (!fn) throw SmobError(SMOB_ERR_CUDA, "cuGreenCtxStreamCreate is not available");
        void* a = nullptr;
        void* b = nullptr;
        if (fn(&a, green, 0x1 /* CU_STREAM_NON_BLOCKING */, prio) != 0 || fn(&b, green, 0x1, far_prio) != 0)
            throw SmobError(SMOB_ERR_CUDA, "cuGreenCtxStreamCreate failed");
        c->st = static_cast<cudaStream_t>(a);
        c->st2 = static_cast<cudaStream_t>(b);
    } else {
        CUDA_OK(cudaStreamCreateWithPriority(&c->st, cudaStreamNonBlocking, prio));
        CUDA_OK(cudaStreamCreateWithPriority(&c->st2, cudaStreamNonBlocking, far_prio));
    }
    c->sh.st = c->st;
    c->sh2.st = c->st2;
    CUDA_OK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CUDA_OK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
}

// the last geometry update rebuilt the grid on the device only: bring the host copy up to date
void refresh_host_grid(const smob_ctx* c) {
    if (!c->host_grid_stale) return;
    set_device(c);
    CUDA_OK(cudaMemcpyAsync(c->coords.data(), c->d_coords.p, sizeof(double) * c->coords.size(), cudaMemcpyDeviceToHost,
                            c->st));
    CUDA_OK(cudaMemcpyAsync(c->norms.data(), c->d_norms.p, sizeof(double) * c->norms.size(), cudaMemcpyDeviceToHost,
                            c->st));
    CUDA_OK(cudaStreamSynchronize(c->st));
    c->host_grid_stale = false;
}

// Orientation after a time step (Sphere::stepEuler, Sphere/Sphere.cpp:367-373, through SimToolbox's
// EquatnHelper::rotateEquatn, which is absent): the rotation by angle |w| dt about w (a lab-frame
// angular velocity) composed on the left, q <- (cos(|w|dt/2), sin(|w|dt/2) w/|w|) q, normalised.
void quat_step(const double* q, const double* w, double dt, double* out) {
    const double wn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (!(wn * std::fabs(dt) > 0)) {
        std::copy(q, q + 4, out);
        return;
    }
    const double h = 0.5 * wn * dt, sh = std::sin(h) / wn;
    const double a0 = std::cos(h), a[3] = {w[0] * sh, w[1] * sh, w[2] * sh};
    // Hamilton product (a0, a) (q0, qv)
    double r[4];
    r[0] = a0 * q[0] - (a[0] * q[1] + a[1] * q[2] + a[2] * q[3]);
    r[1] = a0 * q[1] + q[0] * a[0] + (a[1] * q[3] - a[2] * q[2]);
    r[2] = a0 * q[2] + q[0] * a[1] + (a[2] * q[1] - a[0] * q[3]);
    r[3] = a0 * q[3] + q[0] * a[2] + (a[0] * q[2] - a[1] * q[1]);
    const double n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
    for (int k = 0; k < 4; ++k) out[k] = r[k] / n;
}

// New centres and orientations for the same spheres: near lists and their metadata on the host
// (O(N) data), grid points and far-field copies rebuilt on the device (no host round trip of the
// O(M) arrays). Throws (context unchanged) if spheres of a problem would overlap. The warm-start
// solution is kept; captured graphs and several-RHS copies of the old geometry are dropped.
void update_geometry(smob_ctx* c, const std::vector<double>& centers, const std::vector<double>& quats) {
    {
        DBuf dc;
        dc.upload(centers);
        check_overlap(c, dc.as<double>());  // throws before anything changed
    }
    c->centers = centers;
    c->quats = quats;
    c->d_center.upload(c->centers);
    build_near(c);
    std::vector<char> near_p(kMaxOrder + 1, 0);
    for (int s : c->slot_sphere) near_p[c->orders[s]] = 1;
    bool new_map = false;
    for (int p = 1; p <= kMaxOrder; ++p)
        if (near_p[p] && !(p < (int)c->map_orders.size() && c->map_orders[p])) new_map = true;
    if (new_map) build_tables(c);
    problem_origins(c);
    c->d_center.upload(c->centers);
    c->d_quat.upload(c->quats);
    c->d_org.upload(c->org);
    upload_near(c);
    build_coarse(c);
    bind_geom(c);
    check_launch(c, launch_regrid(c->g, c->d_org.as<double>(), c->st));
    coarse_grids(c);
    c->host_grid_stale = true;
    // (the new geometry may have no coarse targets, so that its FP32 passes run the grid kernels: their
    // tile is tuned by the next solve or operator call, not inside the update)
    c->drop_graphs();
    c->rk = 0;  // recycled solutions belong to the old operator
    for (auto& kv : c->multi) smob_destroy(kv.second);
    c->multi.clear();
    CUDA_OK(cudaStreamSynchronize(c->st));
}

// copy a host 3M vector in, run f(d_in, d_out) with d_out preloaded from host out, copy back
template <typename F>
void host_io(smob_ctx* c, const double* in, double* out, bool load_out, F&& f) {
    const size_t bytes = sizeof(double) * 3 * (size_t)c->M;
    h2d(c, c->d_in.p, in, bytes);
    if (load_out) h2d(c, c->d_out.p, out, bytes);
    else CUDA_OK(cudaMemsetAsync(c->d_out.p, 0, bytes, c->st));
    f(c->d_in.as<double>(), c->d_out.as<double>());
    d2h(c, out, c->d_out.p, bytes);
    check_device_error(c);
}

int op_prec(int precision) {
    if (precision == SMOB_PREC_MIXED) return OP_FP32;
    if (precision == SMOB_PREC_FLOAT_FLOAT) return OP_DF;
    if (precision != SMOB_PREC_FP64) throw SmobError(SMOB_ERR_ARG, "unknown precision");
    return OP_FP64;
}

void all_active(smob_ctx* c) {
    std::vector<unsigned char> a(c->P, 1);
    set_active(c, a);
}

}  // namespace

smob::HostSpheres smob::host_spheres(const smob_ctx* c) {
    refresh_host_grid(c);
    HostSpheres h;
    h.N = c->N;
    h.M = c->M;
    h.centers = c->centers.data();
    h.radii = c->radii.data();
    h.quats = c->quats.data();
    h.coords = c->coords.data();
    h.weights = c->weights.data();
    h.orders = c->orders.data();
    h.gidx = c->gidx.data();
    return h;
}

// ================================================================ C ABI
extern "C" {

const char* smob_last_error(void) { return g_err.c_str(); }

smob_status smob_version(int* major, int* minor) {
    if (major) *major = 0;
    if (minor) *minor = 1;
    return SMOB_OK;
}

smob_status smob_create(smob_ctx** out, const smob_geometry* geo, int device) {
    return smob::create_context(out, geo, device, -1);
}

}  // extern "C"

// Context creation with a stream priority: priority_rank 0 is the device's highest stream
// priority, larger ranks step towards the lowest (two steps per rank: the main stream, then the far
// field's); -1 keeps the default (main stream one step above the far field's). The server gives small
// requests high priority so their kernels are scheduled ahead of large requests' blocks.
smob_status smob::create_context(smob_ctx** out, const smob_geometry* geo, int device, int priority_rank,
                                 void* green_ctx) {
    return guarded([&]() -> smob_status {
        need(out != nullptr && geo != nullptr, "null argument");
        *out = nullptr;
        need(geo->n_spheres > 0, "n_spheres must be positive");
        need(geo->centers && geo->radii && geo->orders, "centers, radii and orders are required");
        need(geo->viscosity > 0 && std::isfinite(geo->viscosity), "viscosity must be positive");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw SmobError(SMOB_ERR_NO_DEVICE, "no CUDA device available");
        }
        need(device >= 0 && device < ndev, "device index out of range");
        std::unique_ptr<smob_ctx> c(new smob_ctx);
        c->device = device;
        CUDA_OK(cudaSetDevice(device));
        int least = 0, greatest = 0;
        CUDA_OK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        // The main stream's chain of small sphere and near-field kernels goes one step ahead of the far
        // field's stream, whose many CTAs fill the SMs that chain leaves free. A ranked context (the
        // server: 0 for its smallest requests) takes the pair of steps 2 rank, 2 rank + 1 from the
        // device's greatest priority (numerically smallest), so every stream of a lower rank stays
        // ahead of both of a higher one's.
        int prio = 0, far_prio = 0;
        if (priority_rank >= 0) {
            prio = std::min(least, greatest + 2 * priority_rank);
            far_prio = std::min(least, greatest + 2 * priority_rank + 1);
        } else {
            prio = std::max(greatest, far_prio - 1);
        }
        create_streams(c.get(), prio, far_prio, green_ctx);
        AllocStreamScope scope(c->st);
        configure_sphere_kernels();
        configure_near_kernels();
        build_context(c.get(), geo);
        ensure_tuned(c.get());
        CUDA_OK(cudaStreamSynchronize(c->st));
        *out = c.release();
        return SMOB_OK;
    });
}

extern "C" {

smob_status smob_destroy(smob_ctx* c) {
    if (!c) return SMOB_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->st);
    delete c;
    return SMOB_OK;
}

smob_status smob_get_sizes(const smob_ctx* c, int* n_spheres, int* n_points, int* n_problems, int* n_near_pairs) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (n_spheres) *n_spheres = c->N;
        if (n_points) *n_points = c->M;
        if (n_problems) *n_problems = c->P;
        if (n_near_pairs) *n_near_pairs = (int)c->nbr_src.size();
        return SMOB_OK;
    });
}

smob_status smob_get_grid(const smob_ctx* c, double* coords, double* norms, double* weights) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (coords || norms) refresh_host_grid(c);
        if (coords) std::copy(c->coords.begin(), c->coords.end(), coords);
        if (norms) std::copy(c->norms.begin(), c->norms.end(), norms);
        if (weights) std::copy(c->weights.begin(), c->weights.end(), weights);
        return SMOB_OK;
    });
}

smob_status smob_set_geometry(smob_ctx* c, const double* centers, const double* quats) {
    return guarded([&]() -> smob_status {
        need(c && centers, "null argument");
        need(c->nrep == 1, "not a user context");
        std::vector<double> ce(centers, centers + 3 * c->N);
        for (double v : ce) need(std::isfinite(v), "centre is not finite");
        std::vector<double> q = c->quats;
        if (quats)
            for (int i = 0; i < c->N; ++i) unit_quat(quats + 4 * i, &q[4 * i], i);
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        update_geometry(c, ce, q);
        return SMOB_OK;
    });
}

smob_status smob_step_euler(smob_ctx* c, const double* vel6n, double dt) {
    return guarded([&]() -> smob_status {
        need(c && vel6n, "null argument");
        need(c->nrep == 1, "not a user context");
        need(std::isfinite(dt), "dt is not finite");
        for (int i = 0; i < 6 * c->N; ++i) need(std::isfinite(vel6n[i]), "velocity is not finite");
        std::vector<double> ce(c->centers), q(c->quats);
        for (int i = 0; i < c->N; ++i) {
            for (int k = 0; k < 3; ++k) ce[3 * i + k] += vel6n[6 * i + k] * dt;
            quat_step(&c->quats[4 * i], vel6n + 6 * i + 3, dt, &q[4 * i]);
        }
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        update_geometry(c, ce, q);
        return SMOB_OK;
    });
}

smob_status smob_get_geometry(const smob_ctx* c, double* centers, double* quats) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (centers) std::copy(c->centers.begin(), c->centers.end(), centers);
        if (quats) std::copy(c->quats.begin(), c->quats.end(), quats);
        return SMOB_OK;
    });
}

smob_status smob_step_euler_device(smob_ctx* c, const double* d_vel6n, double dt) {
    return guarded([&]() -> smob_status {
        need(c && d_vel6n, "null argument");
        CtxScope ctx_scope(c);
        std::vector<double> v(6 * (size_t)c->N);
        d2h(c, v.data(), d_vel6n, sizeof(double) * v.size());
        return smob_step_euler(c, v.data(), dt);
    });
}

smob_status smob_get_near_pairs(const smob_ctx* c, int* trg, int* src) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        int k = 0;
        for (int t = 0; t < c->N; ++t)
            for (int e = c->nbr_start[t]; e < c->nbr_start[t + 1]; ++e, ++k) {
                if (trg) trg[k] = t;
                if (src) src[k] = c->nbr_src[e];
            }
        return SMOB_OK;
    });
}

smob_status smob_coeff_offsets(const smob_ctx* c, int* offsets) {
    return guarded([&]() -> smob_status {
        need(c != nullptr && offsets != nullptr, "null argument");
        for (int i = 0; i < c->N; ++i) offsets[i] = 2 * c->coff[i];
        offsets[c->N] = 2 * c->ncoef_total;
        return SMOB_OK;
    });
}

smob_status smob_apply_p2p(smob_ctx* c, const double* in, double* out, double c_id, double c_sl, double c_trac,
                           int precision) {
    return guarded([&]() -> smob_status {
        need(c && in && out, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        ensure_tuned(c);
        host_io(c, in, out, true, [&](const double* din, double* dout) {
            op_apply(c, din, dout, c_id, c_sl, c_trac, 0.0, op_prec(precision));
        });
        prof_flush(c);
        return SMOB_OK;
    });
}

smob_status smob_apply_lop(smob_ctx* c, const double* in, double* out, double c_lop) {
    return guarded([&]() -> smob_status {
        need(c && in && out, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        host_io(c, in, out, true, [&](const double* din, double* dout) {
            check_launch(c, launch_sphere_op(c->g, din, dout, 0.0, 0.0, -1, c_lop, nullptr, false, c->st));
        });
        return SMOB_OK;
    });
}

smob_status smob_apply(smob_ctx* c, const double* X, double* Y, int n_cols, double alpha, double beta, int precision) {
    return guarded([&]() -> smob_status {
        need(c && X && Y && n_cols >= 1, "invalid argument");
        CtxScope ctx_scope(c);
        all_active(c);
        ensure_tuned(c);
        const size_t n = 3 * (size_t)c->M;
        std::vector<double> tmp(n);
        for (int col = 0; col < n_cols; ++col) {
            host_io(c, X + n * col, tmp.data(), false, [&](const double* din, double* dout) {
                op_apply(c, din, dout, 0.5, 0.0, 1.0, 1.0, op_prec(precision));
            });
            double* y = Y + n * col;
            for (size_t i = 0; i < n; ++i) y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * tmp[i];
        }
        prof_flush(c);
        return SMOB_OK;
    });
}

smob_status smob_project_null_space(smob_ctx* c, double* inout) {
    return guarded([&]() -> smob_status {
        need(c && inout, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        const size_t bytes = sizeof(double) * 3 * (size_t)c->M;
        CUDA_OK(cudaMemcpyAsync(c->d_in.p, inout, bytes, cudaMemcpyHostToDevice, c->st));
        check_launch(c, launch_sh_g2s(c->g, c->d_in.as<double>(), c->d_coef64.as<double>(), c->st));
        check_launch(c, launch_sh_s2g(c->g, c->d_coef64.as<double>(), c->d_out.as<double>(), c->st));
        CUDA_OK(cudaMemcpyAsync(inout, c->d_out.p, bytes, cudaMemcpyDeviceToHost, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_far_field(smob_ctx* c, const double* in, double* out, double c_sl, double c_trac, int precision) {
    return guarded([&]() -> smob_status {
        need(c && in && out, "null argument");
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);  // the fused float-float path allocates its second partial buffer
        all_active(c);
        ensure_tuned(c);
        const bool fp32 = precision == SMOB_PREC_MIXED;
        const bool dfar = precision == SMOB_PREC_FLOAT_FLOAT;
        host_io(c, in, out, true, [&](const double* din, double* dout) {
            const FarItem* items = fp32 ? c->d_items32.as<FarItem>() : c->d_items64.as<FarItem>();
            const int nitems = (int)(fp32 ? c->items32.size() : c->items64.size());
            void* partial = fp32 ? c->d_partial32.p : c->d_partial64.p;
            if (dfar && c_sl != 0.0 && c_trac != 0.0) {
                // both kernels from one float-float pass over the pairs (the mixed solve's fused pass)
                c->d_partial64_sl.alloc(sizeof(double) * c->partial64);
                check_launch(c, launch_far_pack_df(c->g, din, 1.0, c->d_srcdf.as<float4>(), c->st));
                check_launch(c, launch_coarse_src_df(c->g, c->d_srcdf.as<float4>(), c->st));
                const bool hpct = far_df_ct_on(c);
                {
                    ProfScope ps(c, "far_both_df");
                    if (hpct)
                        far_df_ct(c, c->st);
                    else
                        check_launch(c, launch_far_field_df(c->g, c->d_items_df.as<FarItem>(), (int)c->items_df.size(),
                                                            2, c->d_srcdf.as<float4>(), c->d_partial64.as<double>(),
                                                            c->d_partial64_sl.as<double>(), c->st));
                }
                check_launch(c, launch_far_reduce(c->g, c->d_partial64.p, false, c_trac * (-3.0 / (4 * kPi)), dout, c->st,
                                                  hpct ? 2 : 0));
                check_launch(c, launch_far_reduce(c->g, c->d_partial64_sl.p, false, c_sl / (8 * kPi), dout, c->st,
                                                  hpct ? 3 : 0));
                return;
            }
            for (int k = 0; k < 2; ++k) {
                const bool tr = k == 0;
                const double cc = tr ? c_trac : c_sl;
                if (cc == 0.0) continue;
                if (dfar) {
                    check_launch(c, launch_far_pack_df(c->g, din, cc, c->d_srcdf.as<float4>(), c->st));
                    check_launch(c, launch_coarse_src_df(c->g, c->d_srcdf.as<float4>(), c->st));
                    ProfScope ps(c, tr ? "far_trac_df" : "far_sl_df");
                    check_launch(c, launch_far_field_df(c->g, c->d_items_df.as<FarItem>(), (int)c->items_df.size(),
                                                        tr ? 1 : 0, c->d_srcdf.as<float4>(), static_cast<double*>(partial),
                                                        nullptr, c->st));
                } else {
                    check_launch(c, launch_far_pack(c->g, din, cc, c->d_src32.as<float4>(), c->d_src64.as<double4_32a>(), fp32, c->st));
                    if (fp32 && c->g.cs32.ncent > 0) {
                        ProfScope ps(c, "far_coarse");
                        check_launch(c, coarse_src(c, c->st));
                    }
                    if (fp32 && far_ct_on(c)) {
                        far_ct(c, tr, c->st);
                    } else {
                        ProfScope ps(c, fp32 ? (tr ? "far_trac_fp32" : "far_sl_fp32") : (tr ? "far_trac_fp64" : "far_sl_fp64"));
                        check_launch(c, launch_far_field(c->g, items, nitems, tr, fp32, c->d_src32.as<float4>(),
                                                         c->d_src64.as<double4_32a>(), partial, c->st, c->tpt));
                    }
                }
                check_launch(c, launch_far_reduce(c->g, partial, fp32, tr ? -3.0 / (4 * kPi) : 1.0 / (8 * kPi), dout, c->st,
                                                  fp32 && far_ct_on(c) ? 1 : 0));
            }
        });
        prof_flush(c);
        return SMOB_OK;
    });
}

smob_status smob_near_field(smob_ctx* c, const double* in, double* out, double c_sl, double c_trac, int precision) {
    return guarded([&]() -> smob_status {
        need(c && in && out, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        const bool fp32 = precision == SMOB_PREC_MIXED;
        const bool df = precision == SMOB_PREC_FLOAT_FLOAT;  // float-float evaluation of the FP64 sets
        const int nslots = (int)c->slot_sphere.size();
        host_io(c, in, out, true, [&](const double* din, double* dout) {
            if (nslots == 0) return;
            void* coef = fp32 ? c->d_coef32.p : c->d_coef64.p;
            void* sets = fp32 ? c->d_sets32.p : c->d_sets64.p;
            // coefficients only: a sphere pass with no self term and no output contribution
            CUDA_OK(cudaMemsetAsync(c->d_tmp.p, 0, sizeof(double) * 3 * c->M, c->st));
            {
                ProfScope ps(c, "sphere_self");
                check_launch(c, launch_sphere_op(c->g, din, c->d_tmp.as<double>(), 0.0, 0.0, 3, 0.0, coef, fp32, c->st));
            }
            for (int k = 0; k < 2; ++k) {
                const bool tr = k == 0;
                const double cc = tr ? c_trac : c_sl;
                if (cc == 0.0) continue;
                const long long stride = tr ? c->set_stride_trac : c->set_stride_sl;
                {
                    ProfScope ps(c, "near_sets");
                    check_launch(c, launch_near_sets(c->g, coef, tr, fp32, sets, nslots, c->d_slot_sphere.as<int>(),
                                                     stride, c->st, df));
                }
                ProfScope ps(c, tr ? "near_eval_trac" : "near_eval_sl");
                check_launch(c, launch_near_eval(c->g, sets, stride, tr, fp32, cc, dout, c->st, 0, df));
            }
        });
        prof_flush(c);
        return SMOB_OK;
    });
}

smob_status smob_sh_g2s(smob_ctx* c, const double* grid, double* coeff) {
    return guarded([&]() -> smob_status {
        need(c && grid && coeff, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        const size_t bytes = sizeof(double) * 3 * (size_t)c->M;
        CUDA_OK(cudaMemcpyAsync(c->d_in.p, grid, bytes, cudaMemcpyHostToDevice, c->st));
        check_launch(c, launch_sh_g2s(c->g, c->d_in.as<double>(), c->d_coef64.as<double>(), c->st));
        CUDA_OK(cudaMemcpyAsync(coeff, c->d_coef64.p, sizeof(double) * 2 * c->ncoef_total, cudaMemcpyDeviceToHost, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_sh_s2g(smob_ctx* c, const double* coeff, double* grid) {
    return guarded([&]() -> smob_status {
        need(c && grid && coeff, "null argument");
        CtxScope ctx_scope(c);
        all_active(c);
        CUDA_OK(cudaMemcpyAsync(c->d_coef64.p, coeff, sizeof(double) * 2 * c->ncoef_total, cudaMemcpyHostToDevice, c->st));
        check_launch(c, launch_sh_s2g(c->g, c->d_coef64.as<double>(), c->d_out.as<double>(), c->st));
        CUDA_OK(cudaMemcpyAsync(grid, c->d_out.p, sizeof(double) * 3 * c->M, cudaMemcpyDeviceToHost, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

static smob_status check_opts(const smob_solve_opts* o) {
    if (!o) throw SmobError(SMOB_ERR_ARG, "null solve options");
    if (!(o->tol > 0) || o->restart < 1 || o->max_iters < 1) throw SmobError(SMOB_ERR_ARG, "invalid solve options");
    if (o->precision != SMOB_PREC_FP64 && o->precision != SMOB_PREC_MIXED && o->precision != SMOB_PREC_FLOAT_FLOAT)
        throw SmobError(SMOB_ERR_ARG, "unknown precision");
    if (o->precond != 0 && o->precond != 1) throw SmobError(SMOB_ERR_ARG, "unknown preconditioner");
    if (o->warm_start < 0 || o->warm_start > 2) throw SmobError(SMOB_ERR_ARG, "unknown warm start");
    return SMOB_OK;
}

smob_status smob_recycle_info(const smob_ctx* c, int* count, int* capacity) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (count) *count = c->rk;
        if (capacity) *capacity = kRecycleMax;
        return SMOB_OK;
    });
}

smob_status smob_recycle_clear(smob_ctx* c) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        c->rk = 0;
        c->have_xlast = false;
        return SMOB_OK;
    });
}

smob_status smob_solve_mob_device(smob_ctx* c, const double* d_force, double* d_vel, double* d_density,
                                  const smob_solve_opts* o, smob_problem_stats* stats) {
    return guarded([&]() -> smob_status {
        need(c && d_force && d_vel, "null argument");
        check_opts(o);
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        smob_status s = solve_device(c, d_force, d_vel, d_density, o, stats);
        prof_flush(c);
        return s;
    });
}

smob_status smob_solve_mob(smob_ctx* c, const double* force, double* vel, double* density, const smob_solve_opts* o,
                           smob_problem_stats* stats) {
    return guarded([&]() -> smob_status {
        need(c && force && vel, "null argument");
        check_opts(o);
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        for (int i = 0; i < 6 * c->N; ++i)
            if (!std::isfinite(force[i])) throw SmobError(SMOB_ERR_NONFINITE, "force/torque input is not finite");
        ensure_solver(c, std::max(1, o->restart));
        h2d(c, c->d_force.p, force, sizeof(double) * 6 * c->N);
        smob_status s = solve_device(c, c->d_force.as<double>(), c->d_vel.as<double>(),
                                     density ? c->d_out.as<double>() : nullptr, o, stats);
        d2h(c, vel, c->d_vel.p, sizeof(double) * 6 * c->N);
        if (density) d2h(c, density, c->d_out.p, sizeof(double) * 3 * c->M);
        prof_flush(c);
        return s;
    });
}

}  // extern "C"

namespace {
// A child context holding k copies of c's one problem (replica r = problem r), cached per k on c.
// By default the copies form an ordinary batch with c's own far-field settings and kernels: every
// column is then the same bits as its single solve (a problem does not depend on its batch), and the
// batch fills the GPU better than k single solves (cfg2, 8 columns: 117.8 vs 81.7 columns/s). With
// shared pairs (smob_set_multi_shared_pairs) the far field evaluates each grid-point pair once for all
// columns instead (the several-column kernels: grid targets, no float-float compression).
smob_ctx* replicated(smob_ctx* c, int k) {
    auto it = c->multi.find(k);
    if (it != c->multi.end()) return it->second;
    if (c->multi.size() >= 4) {  // bound the cache for callers that cycle through many column counts
        for (auto& kv : c->multi) smob_destroy(kv.second);
        c->multi.clear();
    }
    const int N = c->N;
    std::vector<double> centers, radii, quats;
    std::vector<int> orders, problem;
    for (int r = 0; r < k; ++r) {
        centers.insert(centers.end(), c->centers.begin(), c->centers.end());
        radii.insert(radii.end(), c->radii.begin(), c->radii.end());
        quats.insert(quats.end(), c->quats.begin(), c->quats.end());
        orders.insert(orders.end(), c->orders.begin(), c->orders.end());
        problem.insert(problem.end(), N, r);
    }
    const smob_geometry geo{k * N, centers.data(), radii.data(), quats.data(), orders.data(), problem.data(),
                            c->viscosity};
    std::unique_ptr<smob_ctx> r(new smob_ctx);
    r->device = c->device;
    const bool shared = c->multi_shared;
    r->c32.eps = c->c32.eps;  // replicas share the levels; each column's coarse strengths are its own
    r->c32.ctgt = shared ? false : c->c32.ctgt;  // the several-column kernels evaluate grid targets
    r->chp.eps = shared ? 0.0 : c->chp.eps;      // and every float-float grid-point pair
    r->chp.ctgt = shared ? false : c->chp.ctgt;
    r->eps_hp_auto = shared ? false : c->eps_hp_auto;
    r->coarse_tc = c->coarse_tc;
    r->coarse_interp_tc = c->coarse_interp_tc;
    r->near_tc = c->near_tc;  // the same near and sphere kernels as the single solves (results equal column
    r->sph_tc = c->sph_tc;    // by column)
    CUDA_OK(cudaSetDevice(c->device));
    int least = 0, greatest = 0;
    CUDA_OK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    create_streams(r.get(), std::max(greatest, -1), 0);  // the priorities of a default context
    AllocStreamScope scope(r->st);
    build_context(r.get(), &geo);
    if (shared) {
        r->nrep = k;
        r->rep_M = c->M;
        bind_geom(r.get());  // coarse points per replica
        for (const FarItem& f : r->items_tpt[0])
            if (f.problem == 0) r->items_rep.push_back(f);
        r->d_items_rep.upload(r->items_rep);
    }
    r->use_graphs = c->use_graphs;
    r->loop_graph_on = c->loop_graph_on;
    CUDA_OK(cudaStreamSynchronize(r->st));
    c->multi[k] = r.get();
    return r.release();
}
}  // namespace

extern "C" {

smob_status smob_solve_mob_multi(smob_ctx* c, int n_rhs, const double* force, double* vel, double* density,
                                 const smob_solve_opts* o, smob_problem_stats* stats) {
    return guarded([&]() -> smob_status {
        need(c && force && vel && n_rhs >= 1, "invalid argument");
        need(c->P == 1 && c->nrep == 1, "several right-hand sides need a context with one problem");
        check_opts(o);
        if (n_rhs == 1) return smob_solve_mob(c, force, vel, density, o, stats);
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        smob_ctx* r = replicated(c, n_rhs);
        return smob_solve_mob(r, force, vel, density, o, stats);
    });
}

smob_status smob_mob_apply(smob_ctx* c, const double* X, double* Y, int n_cols, double alpha, double beta,
                           const smob_solve_opts* o) {
    return guarded([&]() -> smob_status {
        need(c && X && Y && n_cols >= 1, "invalid argument");
        const size_t n6 = 6 * (size_t)c->N;
        if (n_cols > 1 && c->P == 1) {
            // all columns in one solve, each with its own Krylov space (SphereSTKMobMat.cpp:129-143
            // solves them one after another)
            std::vector<double> v(n6 * n_cols);
            const smob_status s = smob_solve_mob_multi(c, n_cols, X, v.data(), nullptr, o, nullptr);
            if (s != SMOB_OK && s != SMOB_ERR_NOT_CONVERGED) return s;
            for (size_t i = 0; i < n6 * n_cols; ++i) Y[i] = (beta == 0.0 ? 0.0 : beta * Y[i]) + alpha * v[i];
            return s;
        }
        std::vector<double> v(n6);
        smob_status worst = SMOB_OK;
        for (int col = 0; col < n_cols; ++col) {
            smob_status s = smob_solve_mob(c, X + n6 * col, v.data(), nullptr, o, nullptr);
            if (s != SMOB_OK && s != SMOB_ERR_NOT_CONVERGED) return s;
            if (s != SMOB_OK) worst = s;
            double* y = Y + n6 * col;
            for (size_t i = 0; i < n6; ++i) y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * v[i];
        }
        return worst;
    });
}

smob_status smob_device_alloc(smob_ctx* c, size_t bytes, void** ptr) {
    return guarded([&]() -> smob_status {
        need(c && ptr, "null argument");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaMalloc(ptr, bytes ? bytes : 16));
        return SMOB_OK;
    });
}

smob_status smob_device_free(smob_ctx* c, void* ptr) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        if (ptr) CUDA_OK(cudaFree(ptr));
        return SMOB_OK;
    });
}

smob_status smob_memcpy_h2d(smob_ctx* c, void* dst, const void* src, size_t bytes) {
    return guarded([&]() -> smob_status {
        need(c && dst && src, "null argument");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_memcpy_d2h(smob_ctx* c, void* dst, const void* src, size_t bytes) {
    return guarded([&]() -> smob_status {
        need(c && dst && src, "null argument");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_synchronize(smob_ctx* c) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_profile_enable(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        prof_flush(c);
        c->prof = on != 0;
        return SMOB_OK;
    });
}

smob_status smob_profile_count(const smob_ctx* c, int* n) {
    return guarded([&]() -> smob_status {
        need(c && n, "null argument");
        *n = (int)c->prof_tab.size();
        return SMOB_OK;
    });
}

smob_status smob_profile_get(const smob_ctx* c, int i, char* name, int name_len, long long* launches, double* ms) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        need(i >= 0 && i < (int)c->prof_tab.size(), "profile index out of range");
        auto it = c->prof_tab.begin();
        std::advance(it, i);
        if (name && name_len > 0) {
            std::strncpy(name, it->first.c_str(), name_len - 1);
            name[name_len - 1] = 0;
        }
        if (launches) *launches = it->second.launches;
        if (ms) *ms = it->second.ms;
        return SMOB_OK;
    });
}

smob_status smob_profile_reset(smob_ctx* c) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        prof_flush(c);
        c->prof_tab.clear();
        return SMOB_OK;
    });
}

smob_status smob_launch_count(const smob_ctx* c, long long* launches) {
    return guarded([&]() -> smob_status {
        need(c && launches, "null argument");
        *launches = c->launches;
        return SMOB_OK;
    });
}

smob_status smob_set_graphs(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        c->use_graphs = on != 0;
        if (!c->use_graphs) c->drop_graphs();
        return SMOB_OK;
    });
}

smob_status smob_set_loop_graph(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        c->loop_graph_on = on != 0;
        for (auto& kv : c->multi) smob_set_loop_graph(kv.second, on);
        return SMOB_OK;
    });
}

smob_status smob_loop_graph_info(const smob_ctx* c, int* on, int* available) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (on) *on = c->use_graphs && c->loop_graph_on ? 1 : 0;
        if (available) *available = c->loop_graph_ok ? 1 : 0;
        return SMOB_OK;
    });
}

smob_status smob_launch_stats(const smob_ctx* c, long long* kernels, long long* host_calls) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (kernels) *kernels = c->launches;
        if (host_calls) *host_calls = c->host_calls;
        return SMOB_OK;
    });
}

smob_status smob_tuning(const smob_ctx* c, int* targets_per_thread, double* variant_ms, int* from_cache) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (targets_per_thread) *targets_per_thread = c->tpt;
        if (variant_ms)
            for (int k = 0; k < 3; ++k) variant_ms[k] = c->tune_ms[k];
        if (from_cache) *from_cache = c->tune_cached ? 1 : 0;
        return SMOB_OK;
    });
}

smob_status smob_set_far_compression(smob_ctx* c, double eps, double eps_hp) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        need(std::isfinite(eps) && eps < 1e-3, "far-field tolerance must be below 1e-3 (<= 0: off)");
        need(std::isfinite(eps_hp) && eps_hp <= 1e-9, "float-float far-field tolerance must be at most 1e-9 (<= 0: off)");
        CtxScope ctx_scope(c);
        c->eps_hp_auto = false;  // the caller's choice from now on
        rebuild_far_sets(c, eps, eps_hp);
        return SMOB_OK;
    });
}

smob_status smob_set_far_coarse_targets(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        AllocStreamScope as(c->st);
        c->drop_graphs();  // captured blocks hold the old coarse tables
        for (auto& kv : c->multi) smob_destroy(kv.second);
        c->multi.clear();
        c->c32.ctgt = on != 0;
        c->chp.ctgt = on != 0;
        c->rk = 0;
        build_coarse(c);
        bind_geom(c);
        coarse_grids(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_far_compression_info(const smob_ctx* c, int hp, double* eps, int* coarse_points, int* entries) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        const smob_ctx::CoarseHost& h = hp ? c->chp : c->c32;
        if (eps) *eps = h.eps;
        if (coarse_points) *coarse_points = h.ncoarse;
        if (entries) *entries = (int)h.cent.size();
        return SMOB_OK;
    });
}

smob_status smob_far_pairs(const smob_ctx* c, long long* direct, long long* evaluated, long long* coarse_macs) {
    return smob_far_pairs_set(c, 0, direct, evaluated, coarse_macs);
}

smob_status smob_far_pairs_set(const smob_ctx* c, int hp, long long* direct, long long* evaluated,
                               long long* coarse_macs) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        need(hp == 0 || hp == 1, "hp must be 0 (FP32 set) or 1 (float-float set)");
        // the FP32 kernels' choices replayed on the host for the current work items. With coarse
        // targets, every entry's work items: a candidate counts if its pair takes the entry's level
        // (coarse nodes or the grid points) and is read from the source's level for that target sphere
        // or its grid. Without, the grid items: a source sphere is skipped when every target skips it,
        // read from its grid points when some target needs them, else from the finest coarse level
        // any target votes for. The float-float set (hp = 1) replays the fused float-float pass the same
        // way (its entries, or without coarse targets its votes over items_df).
        const smob_ctx::CoarseHost& h = hp ? c->chp : c->c32;
        const double leps = h.eps > 0 ? std::log(h.eps) : 0.0;
        auto dist = [&](int t, int s) {
            double d2 = 0;
            for (int k = 0; k < 3; ++k) {
                const double dk = c->centers[3 * t + k] - c->centers[3 * s + k];
                d2 += dk * dk;
            }
            return std::sqrt(d2);
        };
        auto near_pair = [&](int t, int s) {
            if (t == s) return true;
            for (int e = c->nbr_start[t]; e < c->nbr_start[t + 1]; ++e)
                if (c->nbr_src[e] == s) return true;
            return false;
        };
        // level index of the source side (nodes on t's surface), -1: grid sources
        auto src_level = [&](int t, int s) {
            const int4* L = &h.clev[(size_t)s * kCoarseLevels];
            if (h.cent.empty() || L[0].x == 0) return -1;
            const double rmin = dist(t, s) - c->radii[t];
            if (!(rmin > c->radii[s])) return -1;
            const double need = leps / std::log(c->radii[s] / rmin) + kCoarseMargin;
            for (int l = 0; l < kCoarseLevels && L[l].x != 0; ++l)
                if (L[l].x >= need) return l;
            return -1;
        };
        // coarse-target level of t for s, -1: grid targets
        auto tgt_lev = [&](int t, int s) {
            const int4* L = &h.clev[(size_t)t * kCoarseLevels];
            if (h.ctent.empty() || L[0].x == 0) return -1;
            const double rmin = dist(t, s) - c->radii[s];
            if (!(rmin > c->radii[t])) return -1;
            const double need = leps / std::log(c->radii[t] / rmin) + kCoarseTargetMargin;
            for (int l = 0; l < kCoarseLevels && L[l].x != 0; ++l)
                if (L[l].x >= need) return L[l].z * kCoarseTargetDen <= c->glen[t] * kCoarseTargetNum ? l : -1;
            return -1;
        };
        long long dir = 0, ev = 0, macs = 0;
        if (!h.ctent.empty()) {
            for (const Problem& pr : c->problems)
                for (int t = pr.s0; t < pr.s1; ++t)
                    for (int s = pr.s0; s < pr.s1; ++s)
                        if (!near_pair(t, s)) dir += (long long)c->glen[t] * c->glen[s];
            // work items of the listed and grid entries: a candidate counts if its pair takes the entry's level
            for (const CtWork& w : h.ct_work) {
                const CtEnt& e = h.ctent[w.ent];
                for (int i = w.sa; i < w.sb; ++i) {
                    const int s = h.ctsrc[i];
                    if (tgt_lev(e.t, s) != e.l) continue;
                    const int lv = src_level(e.t, s);
                    ev += (long long)w.nb * (lv < 0 ? c->glen[s] : h.clev[(size_t)s * kCoarseLevels + lv].z);
                }
            }
            for (const CtEnt& e : h.ctent)
                if (e.l >= 0) macs += 3LL * c->glen[e.t] * e.n;  // interpolation to the grid
        } else {
            std::vector<std::pair<int, int>> tsph;  // (target sphere, targets of it in the item)
            for (const FarItem& it : (hp ? c->items_df : c->items32)) {
                tsph.clear();
                for (int t = it.t0; t < it.t1; ++t) {
                    const int ts = c->sid[t];
                    if (tsph.empty() || tsph.back().first != ts) tsph.push_back({ts, 0});
                    tsph.back().second++;
                }
                for (int s = it.s0; s < it.s1; ++s) {
                    int keep = 0, fine = 0, lvmax = -1;
                    for (auto& ts : tsph) {
                        const int t = ts.first;
                        if (near_pair(t, s)) continue;
                        dir += (long long)ts.second * c->glen[s];
                        keep += ts.second;
                        const int lv = src_level(t, s);
                        if (lv < 0) fine = 1;
                        else lvmax = std::max(lvmax, lv);
                    }
                    if (keep == 0) continue;
                    ev += (long long)keep * (fine ? c->glen[s] : h.clev[(size_t)s * kCoarseLevels + lvmax].z);
                }
            }
        }
        for (const int2& e : h.cent) macs += 3LL * c->glen[e.x] * h.clev[(size_t)e.x * kCoarseLevels + e.y].z;
        if (direct) *direct = dir;
        if (evaluated) *evaluated = ev;
        if (coarse_macs) *coarse_macs = macs;
        return SMOB_OK;
    });
}

smob_status smob_warm_orders(const int* orders, int n_orders) {
    return guarded([&]() -> smob_status {
        need(orders != nullptr || n_orders == 0, "null orders");
        for (int i = 0; i < n_orders; ++i)
            need(orders[i] >= 1 && orders[i] <= kMaxOrder, "orders must lie in 1..32");
        for (int i = 0; i < n_orders; ++i) {
            const int p = orders[i];
            host_tables(p);
            near_map(p, true);
            near_map(p, false);
            for (int pe : kCoarseLadder) {
                if (pe >= p) break;
                coarse_map(p, pe);
                coarse_map_d(p, pe);
            }
        }
        return SMOB_OK;
    });
}

smob_status smob_tc_info(const smob_ctx* c, int* near_tc, int* sphere_tc) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        if (near_tc) *near_tc = c->near_tc ? 1 : 0;
        if (sphere_tc) *sphere_tc = c->sph_tc ? 1 : 0;
        return SMOB_OK;
    });
}

smob_status smob_set_sphere_tc(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        c->drop_graphs();  // captured blocks hold the other kernels
        for (auto& kv : c->multi) smob_set_sphere_tc(kv.second, on);
        c->sph_tc = on != 0;
        c->g.sph_tc = c->sph_tc ? 1 : 0;
        return SMOB_OK;
    });
}

smob_status smob_set_near_tc(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        c->drop_graphs();  // captured blocks hold the other kernel
        for (auto& kv : c->multi) smob_set_near_tc(kv.second, on);
        c->near_tc = on != 0;
        c->g.near_tc = c->near_tc ? 1 : 0;
        // the tile padding must read as zero again after the SIMT layout used the buffer
        CUDA_OK(cudaMemsetAsync(c->d_sets32.p, 0, c->d_sets32.bytes, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_set_coarse_tc(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        c->drop_graphs();  // captured passes hold the other kernel
        need(on >= 0 && on <= 3, "coarse tensor-core mode must be 0-3");
        for (auto& kv : c->multi) smob_set_coarse_tc(kv.second, on);
        c->coarse_tc = on == 1 || on == 2;
        c->coarse_interp_tc = on == 1 || on == 3;
        AllocStreamScope as(c->st);
        coarse_tc_buffers(c, c->c32);
        bind_geom(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_set_multi_shared_pairs(smob_ctx* c, int on) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        CUDA_OK(cudaStreamSynchronize(c->st));
        if ((on != 0) != c->multi_shared) {
            for (auto& kv : c->multi) smob_destroy(kv.second);
            c->multi.clear();
        }
        c->multi_shared = on != 0;
        return SMOB_OK;
    });
}

smob_status smob_coarse_tc_info(const smob_ctx* c, int* on) {
    return guarded([&]() -> smob_status {
        need(c && on, "null argument");
        *on = c->coarse_tc ? (c->coarse_interp_tc ? 1 : 2) : (c->coarse_interp_tc ? 3 : 0);
        return SMOB_OK;
    });
}

smob_status smob_set_far_tile(smob_ctx* c, int targets_per_thread) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        const int k = targets_per_thread == 1 ? 0 : (targets_per_thread == 2 ? 1 : (targets_per_thread == 4 ? 2 : -1));
        need(k >= 0, "targets_per_thread must be 1, 2 or 4");
        CtxScope ctx_scope(c);
        AllocStreamScope as(c->st);
        c->drop_graphs();  // captured blocks hold the old item list and kernel variant
        c->tpt = targets_per_thread;
        c->tuned = true;  // the caller's choice stands
        c->items32 = c->items_tpt[k];
        c->d_items32.upload(c->items32);
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

smob_status smob_timer_mark(smob_ctx* c) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        if (!c->ev_a) {
            CUDA_OK(cudaEventCreate(&c->ev_a));
            CUDA_OK(cudaEventCreate(&c->ev_b));
        }
        CUDA_OK(cudaEventRecord(c->ev_a, c->st));
        return SMOB_OK;
    });
}

smob_status smob_timer_elapsed(smob_ctx* c, double* ms) {
    return guarded([&]() -> smob_status {
        need(c && ms, "null argument");
        need(c->ev_a != nullptr, "smob_timer_mark was not called");
        CUDA_OK(cudaEventRecord(c->ev_b, c->st));
        CUDA_OK(cudaEventSynchronize(c->ev_b));
        float f = 0;
        CUDA_OK(cudaEventElapsedTime(&f, c->ev_a, c->ev_b));
        *ms = f;
        return SMOB_OK;
    });
}

smob_status smob_flush_l2(smob_ctx* c, size_t bytes) {
    return guarded([&]() -> smob_status {
        need(c != nullptr, "null context");
        CtxScope ctx_scope(c);
        AllocStreamScope scope(c->st);
        c->d_flush.alloc(bytes);
        CUDA_OK(cudaMemsetAsync(c->d_flush.p, int(c->flush_val++ & 0xff), bytes, c->st));
        CUDA_OK(cudaStreamSynchronize(c->st));
        return SMOB_OK;
    });
}

}  // extern "C"

