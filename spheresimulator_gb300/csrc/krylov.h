// krylov.h — batched GMRES kernels (see krylov.cu).
#pragma once
#include "smob_internal.h"

namespace smob {

struct VecChunk {
    long long l0, l1;  // element range, inside one problem's segment
    int problem;
    int pad;
};

// per-problem Krylov state kept on the device
struct KrylovState {
    double tol_abs;    // cycle stop threshold on the implicit residual |g_{j+1}|
    int kcount;        // Krylov vectors built in the current cycle
    int iters;         // total GMRES iterations
    int cycle_fp32;    // 1 when the current cycle applies the FP32 operator
    int passes32;      // operator applications, FP32
    int passes64;      // operator applications, FP64 (inner iterations only; host adds the rest)
    int nonfinite;     // NaN/Inf met
};

// elementwise kernels: grid (chunk, kElemBlocks) of kElemThreads threads, one element per thread
constexpr int kElemThreads = 256;
constexpr int kElemBlocks = kVecChunk / kElemThreads;

struct KrylovLaunch {
    const VecChunk* chunks;
    int nchunks;
    const Problem* problems;
    int P;
    double* partial;  // nchunks * max_nvec
    long long partial_cap;  // doubles in partial
    unsigned* counters;  // P * cstride, zero between launches (launch_dots' last chunk of each sum resets it)
    int cstride;         // counters per problem (the most vectors one launch_dots may take)
};

// out[p*ostride + ooff + i] (+)= <A_i, b> over problem p's segment for i < nvec (sqrt if take_sqrt);
// out2 (optional) receives the same values at out2[p*ostride2 + i] (accumulated if accumulate2)
int launch_dots(const KrylovLaunch& L, const double* A, long long lda, int nvec, const double* b,
                const unsigned char* active, double* out, long long ostride, long long ooff, bool accumulate,
                bool take_sqrt, cudaStream_t st, double* out2 = nullptr, long long ostride2 = 0,
                bool accumulate2 = false);
int launch_update(const KrylovLaunch& L, const double* V, long long ldv, int nvec, const int* nvec_p, const double* h,
                  long long hstride, double sign, const unsigned char* active, double* w, cudaStream_t st);
int launch_scale(const KrylovLaunch& L, const double* src, const double* val, long long vstride, bool invert,
                 const unsigned char* active, double* dst, cudaStream_t st);
int launch_axpby_seg(const KrylovLaunch& L, double a, const double* x, double b, const unsigned char* active, double* y,
                     cudaStream_t st);
int launch_cycle_init(const KrylovLaunch& L, int m, const unsigned char* in_cycle, const double* beta, KrylovState* ks,
                      double* H, double* g, cudaStream_t st);
// The second CGS2 update of an Arnoldi step fused with what follows it: w -= V h (as launch_update
// with sign -1), |w| into hnorm, and the Givens step of column j (rotations, g, the stop test), the last two by the
// last CTA of each problem. Needs nchunks * kElemBlocks partials; returns -1 if L.partial is smaller.
int launch_update_norm_givens(const KrylovLaunch& L, const double* V, long long ldv, int nvec, const double* h,
                              long long hstride, unsigned char* active, double* w, double* hnorm, int j, int m,
                              KrylovState* ks, double* H, double* g, double* cs, double* sn, int maxit,
                              cudaStream_t st);
int launch_trisolve(const KrylovLaunch& L, int m, const unsigned char* in_cycle, const KrylovState* ks, const double* H,
                    const double* g, double* y, int* kc, cudaStream_t st);

// ---- device-side control of the restart-cycle loop (graph-driven solve)
// The loop's decisions, taken on the host between Krylov blocks otherwise, run as single-CTA kernels
// inside one CUDA graph and steer its conditional nodes (while / switch / if). These kernels call
// cudaGraphSetConditional, so they may only run as nodes of such a graph.

// per-problem solve state, device-resident while the graph runs
struct SolveTrack {
    double bnorm;       // |b|
    double beta;        // current residual norm (high precision, or updated from one by an FP32 step)
    int done, conv;     // finished; converged
    int hp_now;         // beta is (derived from) a high-precision residual: it may end the solve
    int hp_done;        // a high-precision residual after a cycle exists (u_hp, x_hp are valid)
    int x_moved;        // x changed since the last high-precision residual
    int cycles;         // restart cycles run
    int passes64;       // high-precision operator passes outside the Arnoldi steps
    int passes32x;      // FP32 operator passes outside the Arnoldi steps
};

// the solve's scalars and the loop's body counters (bodies run, for the kernel count)
struct SolveParams {
    double tol, inner_tol;
    int mixed;
    int max_cycles;  // bound on the cycles of one launch: every cycle advances each of its problems by one
                     // iteration at least, so more than the iteration limit means a broken loop
    int cycles_run, upd_run, hp_run;
    int overrun;     // set when the bound stopped the loop (the solve's results are void)
    int fin_from, fin_moved, fin_fresh;  // full-solve graph: final-velocity bodies run
    int pad;
};

// next cycle: (merge) beta of the problems of the cycle that ended = norm; then per problem: stop
// (converged / iteration limit / non-finite) or join the cycle (in_cycle, active, the cycle's stop
// threshold in ks); beta_out = beta; while-handle = any problem in the cycle
int launch_loop_decide(int P, bool merge, SolveTrack* t, KrylovState* ks, SolveParams* sp, const double* norm,
                       unsigned char* in_cycle, unsigned char* active, double* beta_out, int maxit,
                       unsigned long long h_cycle, cudaStream_t st);
// start of the Arnoldi steps of a cycle: step counter 0, inner while-handle 1 (the switch handle is
// already 0: its default, and the last step of the previous cycle resets it)
int launch_inner_begin(int* jdev, unsigned long long h_inner, cudaStream_t st);
// after step j: counts it; the next step runs (switch-handle j+1) while a problem is active and
// j+1 < m, otherwise the inner loop ends and the switch handle goes back to 0
int launch_step_next(int P, const unsigned char* active, int* jdev, int* runs_j, int m, unsigned long long h_inner,
                     unsigned long long h_sel, cudaStream_t st);
// residual of the cycle's problems: FP32 update (MIXED, a high-precision residual exists and
// beta <= 1e-4 |b|) or a high-precision residual; masks and if-handles for both
int launch_resid_decide(int P, const SolveTrack* t, SolveParams* sp, const unsigned char* in_cycle, unsigned char* upd,
                        unsigned char* hpm, unsigned long long h_upd, unsigned long long h_hp, cudaStream_t st);
// bookkeeping of a residual pass on the problems in mask: kind 0 FP32 update, kind 1 high precision
int launch_track_mark(int P, SolveTrack* t, const unsigned char* mask, int kind, cudaStream_t st);
// cold start of the full-solve graph: the per-problem state from |b| and |r| (non-finite: stopped;
// |b| < 1e-5: converged, zero correction), the set-up pass counted in the solve's precision
int launch_track_init(int P, bool mixed, const double* bnorm, const double* rnorm, SolveTrack* t, cudaStream_t st);
// final velocity of the full-solve graph: per problem u from u_hp (MIXED with a high-precision
// residual; plus the FP32 single layer of x - x_hp where x moved since) or a fresh high-precision
// single-layer pass; masks and if-handles, pass counts
int launch_final_decide(int P, SolveTrack* t, SolveParams* sp, unsigned char* from_hp, unsigned char* moved,
                        unsigned char* fresh, unsigned long long h_from, unsigned long long h_moved,
                        unsigned long long h_fresh, cudaStream_t st);

}  // namespace smob
