// krylov.cu — device-side restarted GMRES building blocks for a batch of independent problems.
//
// Replaces the Belos pseudo-block GMRES that SphereSTKMobMat drives (BIE/SphereSTKMobMat.cpp:55-61,
// 209-241; settings in mobilitySolver.yaml:3-16). Every vector of the batch is the concatenation
// of the problems' segments; reductions run over fixed chunks that never cross a problem
// boundary and are finalised in a fixed order, so each problem's arithmetic is the same alone
// or inside any batch. Orthogonalisation is classical Gram-Schmidt applied twice (CGS2), which
// gives the same Krylov basis to rounding as the reference's iterated modified Gram-Schmidt
// while needing two reductions per pass instead of j+1 dependent ones.
#include "krylov.h"

namespace smob {

namespace {

__device__ __forceinline__ double block_reduce(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; ++i) s += red[i];
    }
    return s;
}

// Chunk dot products <A_i, b> with the final sum fused in: every CTA writes its chunk's partial, and
// the last CTA of a (problem, vector) to finish (a counter per pair, after a memory fence) adds that
// problem's partials (thread t every blockDim.x-th chunk from t on, then the block's fixed reduction
// tree) and writes out[p*ostride + ooff + i] (+)= sum (sqrt if take_sqrt; optionally also out2), then
// resets the counter. The order of the final sum is fixed, so the result does not depend on which CTA
// finishes last.
__global__ void k_chunk_dots(const VecChunk* __restrict__ chunks, const double* __restrict__ A, long long lda,
                             const double* __restrict__ b, const unsigned char* __restrict__ active,
                             double* __restrict__ partial, int nchunks, const Problem* __restrict__ probs,
                             unsigned* __restrict__ counters, int cstride, double* out, long long ostride,
                             long long ooff, int accumulate, int take_sqrt, double* out2, long long ostride2,
                             int accumulate2) {
    __shared__ double red[32];
    const VecChunk ch = chunks[blockIdx.x];
    if (active && !active[ch.problem]) return;
    const int i = blockIdx.y;
    const double* a = A + lda * i;
    double s = 0;
    for (long long l = ch.l0 + threadIdx.x; l < ch.l1; l += blockDim.x) s = fma(a[l], b[l], s);
    s = block_reduce(s, red);
    __shared__ int last;
    const Problem pr = probs[ch.problem];
    unsigned* cnt = counters + (long long)ch.problem * cstride + i;
    if (threadIdx.x == 0) {
        partial[(long long)i * nchunks + blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(cnt, 1u) == (unsigned)(pr.c1 - pr.c0 - 1);
    }
    __syncthreads();
    if (!last) return;  // CTA-uniform
    // the last chunk of this (problem, vector): every partial is written
    __threadfence();
    double t = 0;
    for (int c = pr.c0 + threadIdx.x; c < pr.c1; c += blockDim.x) t += __ldcg(partial + (long long)i * nchunks + c);
    t = block_reduce(t, red);
    if (threadIdx.x != 0) return;
    *cnt = 0u;
    if (take_sqrt) t = sqrt(t);
    double* o = out + ostride * ch.problem + ooff + i;
    *o = accumulate ? *o + t : t;
    if (out2) {
        double* o2 = out2 + ostride2 * ch.problem + i;
        *o2 = accumulate2 ? *o2 + t : t;
    }
}

// Elementwise kernels: grid (chunk, kElemBlocks), one element per thread, so a small problem's
// few chunks still spread over the whole GPU. Per element the arithmetic is independent of the grid.

// w[l] += sign * sum_{i < n_p} h[p*hstride + i] * V[i*ldv + l]
__global__ void k_chunk_update(const VecChunk* __restrict__ chunks, const double* __restrict__ V, long long ldv,
                               int nvec, const int* __restrict__ nvec_p, const double* __restrict__ h,
                               long long hstride, double sign, const unsigned char* __restrict__ active,
                               double* __restrict__ w) {
    const VecChunk ch = chunks[blockIdx.x];
    if (active && !active[ch.problem]) return;
    const long long l = ch.l0 + (long long)blockIdx.y * kElemThreads + threadIdx.x;
    if (l >= ch.l1) return;
    const int n = nvec_p ? nvec_p[ch.problem] : nvec;
    const double* hp = h + hstride * ch.problem;
    double s = 0;
    for (int i = 0; i < n; ++i) s = fma(hp[i], V[ldv * i + l], s);
    w[l] = fma(sign, s, w[l]);
}

// dst[l] = src[l] * f(p) with f = 1/val[p] (invert) or val[p]
__global__ void k_chunk_scale(const VecChunk* __restrict__ chunks, const double* __restrict__ src,
                              const double* __restrict__ val, long long vstride, int invert,
                              const unsigned char* __restrict__ active, double* __restrict__ dst) {
    const VecChunk ch = chunks[blockIdx.x];
    if (active && !active[ch.problem]) return;
    const long long l = ch.l0 + (long long)blockIdx.y * kElemThreads + threadIdx.x;
    if (l >= ch.l1) return;
    double f = val[vstride * ch.problem];
    if (invert) f = f != 0 ? 1.0 / f : 0.0;
    dst[l] = src[l] * f;
}

// y = a*x + b*y on active problems (b == 0 overwrites)
__global__ void k_chunk_axpby(const VecChunk* __restrict__ chunks, double a, const double* __restrict__ x, double b,
                              const unsigned char* __restrict__ active, double* __restrict__ y) {
    const VecChunk ch = chunks[blockIdx.x];
    if (active && !active[ch.problem]) return;
    const long long l = ch.l0 + (long long)blockIdx.y * kElemThreads + threadIdx.x;
    if (l >= ch.l1) return;
    y[l] = (b == 0.0) ? a * x[l] : fma(a, x[l], b * y[l]);
}

__global__ void k_cycle_init(int P, int m, const unsigned char* __restrict__ in_cycle, const double* __restrict__ beta,
                             KrylovState* __restrict__ ks, double* __restrict__ H, double* __restrict__ gv) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !in_cycle[p]) return;
    double* Hp = H + (long long)p * m * (m + 1);
    for (int i = 0; i < m * (m + 1); ++i) Hp[i] = 0;
    double* g = gv + (long long)p * (m + 1);
    for (int i = 0; i <= m; ++i) g[i] = 0;
    g[0] = beta[p];
    ks[p].kcount = 0;
}

// Givens step of column j for problem p: rotate H[:, j] by the previous rotations, make the new one
// from (H[j, j], hn), update g and the per-problem stop test
__device__ void givens_one(int p, int j, int m, KrylovState* __restrict__ ks, double* __restrict__ H,
                           double* __restrict__ gv, double* __restrict__ cs, double* __restrict__ sn, double hn,
                           unsigned char* __restrict__ active, int maxit) {
    double* Hc = H + (long long)p * m * (m + 1) + (long long)j * (m + 1);
    double* c = cs + (long long)p * m;
    double* s = sn + (long long)p * m;
    double* g = gv + (long long)p * (m + 1);
    Hc[j + 1] = hn;
    for (int i = 0; i < j; ++i) {
        const double a = Hc[i], b = Hc[i + 1];
        Hc[i] = c[i] * a + s[i] * b;
        Hc[i + 1] = -s[i] * a + c[i] * b;
    }
    const double a = Hc[j], b = Hc[j + 1];
    const double d = hypot(a, b);
    c[j] = d > 0 ? a / d : 1.0;
    s[j] = d > 0 ? b / d : 0.0;
    Hc[j] = d;
    Hc[j + 1] = 0;
    g[j + 1] = -s[j] * g[j];
    g[j] = c[j] * g[j];
    KrylovState& k = ks[p];
    k.kcount = j + 1;
    k.iters += 1;
    k.passes32 += k.cycle_fp32;
    k.passes64 += 1 - k.cycle_fp32;
    const bool finite = isfinite(g[j + 1]) && isfinite(hn);
    if (!finite) k.nonfinite = 1;
    if (!finite || fabs(g[j + 1]) < k.tol_abs || hn == 0.0 || j + 1 == m || k.iters >= maxit) active[p] = 0;
}

// w[l] -= sum_{i < nvec} h[p*hstride + i] * V[i*ldv + l] (the arithmetic of k_chunk_update), then |w|^2
// per CTA into partial[chunk * kElemBlocks + blockIdx.y]; the last CTA of a problem (a counter per
// problem, after a memory fence) adds the problem's partials, thread t taking every kElemThreads-th one
// from t on, then the block's fixed reduction tree; thread 0 writes hnorm[p] = sqrt of the sum, resets
// the counter and runs the Givens step of column j. The final sum's order is fixed, so the result does
// not depend on which CTA finishes last.
__global__ void __launch_bounds__(kElemThreads)
    k_chunk_update_norm_givens(const VecChunk* __restrict__ chunks, const Problem* __restrict__ probs,
                               const double* __restrict__ V, long long ldv, int nvec, const double* __restrict__ h,
                               long long hstride, unsigned char* __restrict__ active, double* __restrict__ w,
                               double* __restrict__ partial, unsigned* __restrict__ counters, int cstride,
                               double* __restrict__ hnorm, int j, int m, KrylovState* __restrict__ ks,
                               double* __restrict__ H, double* __restrict__ gv, double* __restrict__ cs,
                               double* __restrict__ sn, int maxit) {
    __shared__ double red[kElemThreads / 32];
    const VecChunk ch = chunks[blockIdx.x];
    if (!active[ch.problem]) return;  // CTA-uniform
    const long long l = ch.l0 + (long long)blockIdx.y * kElemThreads + threadIdx.x;
    double sq = 0;
    if (l < ch.l1) {
        const double* hp = h + hstride * ch.problem;
        double s = 0;
        for (int i = 0; i < nvec; ++i) s = fma(hp[i], V[ldv * i + l], s);
        const double v = fma(-1.0, s, w[l]);
        w[l] = v;
        sq = v * v;
    }
    sq = block_reduce(sq, red);
    __shared__ int last;
    const Problem pr = probs[ch.problem];
    unsigned* cnt = counters + (long long)ch.problem * cstride;
    if (threadIdx.x == 0) {
        partial[(long long)blockIdx.x * kElemBlocks + blockIdx.y] = sq;
        __threadfence();
        last = atomicAdd(cnt, 1u) == (unsigned)((pr.c1 - pr.c0) * kElemBlocks - 1);
    }
    __syncthreads();
    if (!last) return;  // CTA-uniform
    // the last CTA of this problem: every partial is written
    __threadfence();
    double t = 0;
    for (long long q = (long long)pr.c0 * kElemBlocks + threadIdx.x; q < (long long)pr.c1 * kElemBlocks;
         q += kElemThreads)
        t += __ldcg(partial + q);
    t = block_reduce(t, red);
    if (threadIdx.x != 0) return;
    *cnt = 0u;
    const double hn = sqrt(t);
    hnorm[ch.problem] = hn;
    givens_one(ch.problem, j, m, ks, H, gv, cs, sn, hn, active, maxit);
}

__global__ void k_trisolve(int P, int m, const unsigned char* __restrict__ in_cycle, const KrylovState* __restrict__ ks,
                           const double* __restrict__ H, const double* __restrict__ gv, double* __restrict__ y) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !in_cycle[p]) return;
    const int k = ks[p].kcount;
    const double* Hp = H + (long long)p * m * (m + 1);
    const double* g = gv + (long long)p * (m + 1);
    double* yp = y + (long long)p * m;
    for (int i = k - 1; i >= 0; --i) {
        double t = g[i];
        for (int l = i + 1; l < k; ++l) t -= Hp[(long long)l * (m + 1) + i] * yp[l];
        const double d = Hp[(long long)i * (m + 1) + i];
        yp[i] = d != 0 ? t / d : 0.0;
    }
    for (int i = k; i < m; ++i) yp[i] = 0;
}

__global__ void k_kcount(int P, const KrylovState* __restrict__ ks, int* __restrict__ kc) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) kc[p] = ks[p].kcount;
}

// ---- loop control (one CTA; thread 0 alone sets the conditional handles)
constexpr int kCtlThreads = 256;

// The per-problem rules are those of the host-driven loop in api.cu, operation for operation, so
// both loops take the same decisions on the same values.
__global__ void k_loop_decide(int P, int merge, SolveTrack* __restrict__ t, KrylovState* __restrict__ ks,
                              SolveParams* __restrict__ sp, const double* __restrict__ norm,
                              unsigned char* __restrict__ in_cycle, unsigned char* __restrict__ active,
                              double* __restrict__ beta_out, int maxit, cudaGraphConditionalHandle h_cycle) {
    const double tol = sp->tol, inner_tol = sp->inner_tol;
    const int mixed = sp->mixed;
    int any = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        SolveTrack tr = t[p];
        if (merge && in_cycle[p]) tr.beta = norm[p];
        unsigned char cyc = 0;
        if (!tr.done) {
            if (tr.beta / tr.bnorm < tol && tr.hp_now) {
                tr.done = 1;
                tr.conv = 1;
            } else if (ks[p].iters >= maxit || ks[p].nonfinite) {
                tr.done = 1;
            } else {
                cyc = 1;
                tr.cycles += 1;
                const double a = __dmul_rn(inner_tol, tr.beta), b = __dmul_rn(__dmul_rn(0.5, tol), tr.bnorm);
                ks[p].tol_abs = mixed ? (a < b ? b : a) : __dmul_rn(tol, tr.bnorm);
                ks[p].cycle_fp32 = mixed ? 1 : 0;
            }
        }
        in_cycle[p] = cyc;
        active[p] = cyc;
        beta_out[p] = tr.beta;
        t[p] = tr;
        any |= cyc;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        if (any && sp->cycles_run >= sp->max_cycles) {
            sp->overrun = 1;
            any = 0;
        }
        if (any) sp->cycles_run += 1;
        cudaGraphSetConditional(h_cycle, any ? 1u : 0u);
    }
}

__global__ void k_inner_begin(int* __restrict__ jdev, cudaGraphConditionalHandle h_inner) {
    if (threadIdx.x == 0) {
        *jdev = 0;
        cudaGraphSetConditional(h_inner, 1u);
    }
}

__global__ void k_step_next(int P, const unsigned char* __restrict__ active, int* __restrict__ jdev,
                            int* __restrict__ runs_j, int m, cudaGraphConditionalHandle h_inner,
                            cudaGraphConditionalHandle h_sel) {
    int any = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) any |= active[p] ? 1 : 0;
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        const int j = *jdev;
        runs_j[j] += 1;
        const int next = j + 1;
        *jdev = next;
        const bool more = any && next < m;
        cudaGraphSetConditional(h_sel, more ? (unsigned)next : 0u);
        cudaGraphSetConditional(h_inner, more ? 1u : 0u);
    }
}

__global__ void k_resid_decide(int P, const SolveTrack* __restrict__ t, SolveParams* __restrict__ sp,
                               const unsigned char* __restrict__ in_cycle, unsigned char* __restrict__ upd,
                               unsigned char* __restrict__ hpm, cudaGraphConditionalHandle h_upd,
                               cudaGraphConditionalHandle h_hp) {
    const int mixed = sp->mixed;
    int any_u = 0, any_h = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        unsigned char u = 0, h = 0;
        if (in_cycle[p]) {
            const SolveTrack tr = t[p];
            if (mixed && tr.hp_done && tr.beta <= __dmul_rn(1e-4, tr.bnorm)) u = 1;
            else h = 1;
        }
        upd[p] = u;
        hpm[p] = h;
        any_u |= u;
        any_h |= h;
    }
    any_u = __syncthreads_or(any_u);
    any_h = __syncthreads_or(any_h);
    if (threadIdx.x == 0) {
        if (any_u) sp->upd_run += 1;
        if (any_h) sp->hp_run += 1;
        cudaGraphSetConditional(h_upd, any_u ? 1u : 0u);
        cudaGraphSetConditional(h_hp, any_h ? 1u : 0u);
    }
}

__global__ void k_track_init(int P, int mixed, const double* __restrict__ bnorm, const double* __restrict__ rnorm,
                             SolveTrack* __restrict__ t) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    SolveTrack tr;
    tr.bnorm = bnorm[p];
    tr.beta = rnorm[p];
    tr.done = 0;
    tr.conv = 0;
    if (!isfinite(tr.bnorm) || !isfinite(tr.beta)) {
        tr.done = 1;
    } else if (tr.bnorm < 1e-5) {  // forcing is zero: density correction is zero (SphereSTKMobMat.cpp:217)
        tr.done = 1;
        tr.conv = 1;
    }
    tr.hp_now = mixed ? 0 : 1;
    tr.hp_done = 0;
    tr.x_moved = 0;
    tr.cycles = 0;
    tr.passes64 = mixed ? 0 : 1;
    tr.passes32x = mixed ? 1 : 0;
    t[p] = tr;
}

__global__ void k_final_decide(int P, SolveTrack* __restrict__ t, SolveParams* __restrict__ sp,
                               unsigned char* __restrict__ from_hp, unsigned char* __restrict__ moved,
                               unsigned char* __restrict__ fresh, cudaGraphConditionalHandle h_from,
                               cudaGraphConditionalHandle h_moved, cudaGraphConditionalHandle h_fresh) {
    const int mixed = sp->mixed;
    int any_f = 0, any_m = 0, any_r = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        SolveTrack& tr = t[p];
        const unsigned char f = (mixed && tr.hp_done) ? 1 : 0;
        const unsigned char mv = (f && tr.x_moved) ? 1 : 0;
        const unsigned char fr = f ? 0 : 1;
        if (mv) tr.passes32x += 1;
        if (fr) tr.passes64 += 1;
        from_hp[p] = f;
        moved[p] = mv;
        fresh[p] = fr;
        any_f |= f;
        any_m |= mv;
        any_r |= fr;
    }
    any_f = __syncthreads_or(any_f);
    any_m = __syncthreads_or(any_m);
    any_r = __syncthreads_or(any_r);
    if (threadIdx.x == 0) {
        sp->fin_from = any_f ? 1 : 0;
        sp->fin_moved = any_m ? 1 : 0;
        sp->fin_fresh = any_r ? 1 : 0;
        cudaGraphSetConditional(h_from, any_f ? 1u : 0u);
        cudaGraphSetConditional(h_moved, any_m ? 1u : 0u);
        cudaGraphSetConditional(h_fresh, any_r ? 1u : 0u);
    }
}

__global__ void k_track_mark(int P, SolveTrack* __restrict__ t, const unsigned char* __restrict__ mask, int kind) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !mask[p]) return;
    SolveTrack& tr = t[p];
    if (kind == 0) {
        tr.passes32x += 1;
        tr.x_moved = 1;
    } else {
        tr.passes64 += 1;
        tr.hp_done = 1;
        tr.hp_now = 1;
        tr.x_moved = 0;
    }
}

}  // namespace

int launch_dots(const KrylovLaunch& L, const double* A, long long lda, int nvec, const double* b,
                const unsigned char* active, double* out, long long ostride, long long ooff, bool accumulate,
                bool take_sqrt, cudaStream_t st, double* out2, long long ostride2, bool accumulate2) {
    if (nvec > L.cstride) return -1;  // more vectors than counters per problem
    dim3 grid(L.nchunks, nvec);
    k_chunk_dots<<<grid, 256, 0, st>>>(L.chunks, A, lda, b, active, L.partial, L.nchunks, L.problems, L.counters,
                                       L.cstride, out, ostride, ooff, accumulate ? 1 : 0, take_sqrt ? 1 : 0, out2,
                                       ostride2, accumulate2 ? 1 : 0);
    return 1;
}

int launch_update(const KrylovLaunch& L, const double* V, long long ldv, int nvec, const int* nvec_p, const double* h,
                  long long hstride, double sign, const unsigned char* active, double* w, cudaStream_t st) {
    k_chunk_update<<<dim3(L.nchunks, kElemBlocks), kElemThreads, 0, st>>>(L.chunks, V, ldv, nvec, nvec_p, h, hstride,
                                                                          sign, active, w);
    return 1;
}

int launch_scale(const KrylovLaunch& L, const double* src, const double* val, long long vstride, bool invert,
                 const unsigned char* active, double* dst, cudaStream_t st) {
    k_chunk_scale<<<dim3(L.nchunks, kElemBlocks), kElemThreads, 0, st>>>(L.chunks, src, val, vstride, invert ? 1 : 0,
                                                                         active, dst);
    return 1;
}

int launch_axpby_seg(const KrylovLaunch& L, double a, const double* x, double b, const unsigned char* active, double* y,
                     cudaStream_t st) {
    k_chunk_axpby<<<dim3(L.nchunks, kElemBlocks), kElemThreads, 0, st>>>(L.chunks, a, x, b, active, y);
    return 1;
}

int launch_cycle_init(const KrylovLaunch& L, int m, const unsigned char* in_cycle, const double* beta, KrylovState* ks,
                      double* H, double* g, cudaStream_t st) {
    k_cycle_init<<<(L.P + 63) / 64, 64, 0, st>>>(L.P, m, in_cycle, beta, ks, H, g);
    return 1;
}

int launch_update_norm_givens(const KrylovLaunch& L, const double* V, long long ldv, int nvec, const double* h,
                              long long hstride, unsigned char* active, double* w, double* hnorm, int j, int m,
                              KrylovState* ks, double* H, double* g, double* cs, double* sn, int maxit,
                              cudaStream_t st) {
    if ((long long)L.nchunks * kElemBlocks > L.partial_cap || L.cstride < 1) return -1;
    k_chunk_update_norm_givens<<<dim3(L.nchunks, kElemBlocks), kElemThreads, 0, st>>>(
        L.chunks, L.problems, V, ldv, nvec, h, hstride, active, w, L.partial, L.counters, L.cstride, hnorm, j, m, ks,
        H, g, cs, sn, maxit);
    return 1;
}

int launch_trisolve(const KrylovLaunch& L, int m, const unsigned char* in_cycle, const KrylovState* ks, const double* H,
                    const double* g, double* y, int* kc, cudaStream_t st) {
    k_trisolve<<<(L.P + 63) / 64, 64, 0, st>>>(L.P, m, in_cycle, ks, H, g, y);
    k_kcount<<<(L.P + 63) / 64, 64, 0, st>>>(L.P, ks, kc);
    return 2;
}

int launch_loop_decide(int P, bool merge, SolveTrack* t, KrylovState* ks, SolveParams* sp, const double* norm,
                       unsigned char* in_cycle, unsigned char* active, double* beta_out, int maxit,
                       unsigned long long h_cycle, cudaStream_t st) {
    k_loop_decide<<<1, kCtlThreads, 0, st>>>(P, merge ? 1 : 0, t, ks, sp, norm, in_cycle, active, beta_out, maxit,
                                             h_cycle);
    return 1;
}

int launch_inner_begin(int* jdev, unsigned long long h_inner, cudaStream_t st) {
    k_inner_begin<<<1, 32, 0, st>>>(jdev, h_inner);
    return 1;
}

int launch_step_next(int P, const unsigned char* active, int* jdev, int* runs_j, int m, unsigned long long h_inner,
                     unsigned long long h_sel, cudaStream_t st) {
    k_step_next<<<1, kCtlThreads, 0, st>>>(P, active, jdev, runs_j, m, h_inner, h_sel);
    return 1;
}

int launch_resid_decide(int P, const SolveTrack* t, SolveParams* sp, const unsigned char* in_cycle, unsigned char* upd,
                        unsigned char* hpm, unsigned long long h_upd, unsigned long long h_hp, cudaStream_t st) {
    k_resid_decide<<<1, kCtlThreads, 0, st>>>(P, t, sp, in_cycle, upd, hpm, h_upd, h_hp);
    return 1;
}

int launch_track_init(int P, bool mixed, const double* bnorm, const double* rnorm, SolveTrack* t, cudaStream_t st) {
    k_track_init<<<(P + 127) / 128, 128, 0, st>>>(P, mixed ? 1 : 0, bnorm, rnorm, t);
    return 1;
}

int launch_final_decide(int P, SolveTrack* t, SolveParams* sp, unsigned char* from_hp, unsigned char* moved,
                        unsigned char* fresh, unsigned long long h_from, unsigned long long h_moved,
                        unsigned long long h_fresh, cudaStream_t st) {
    k_final_decide<<<1, kCtlThreads, 0, st>>>(P, t, sp, from_hp, moved, fresh, h_from, h_moved, h_fresh);
    return 1;
}

int launch_track_mark(int P, SolveTrack* t, const unsigned char* mask, int kind, cudaStream_t st) {
    k_track_mark<<<(P + 127) / 128, 128, 0, st>>>(P, t, mask, kind);
    return 1;
}

}  // namespace smob
