// near.cu — spectral near-field evaluation for near sphere pairs.
//
// Replaces NearEvaluator::operator() (BIE/SphereSTKSHOperator.cpp:575-695), driven by the
// neighbour list that MPI/NearInteraction.txx:430-447 builds (pairs (t,s), t != s,
// |c_s - c_t| < 1.5 (a_s + a_t)). The reference adds cTrac*(KL_spectral - direct) at the
// target's grid points; the far-field kernel here never adds the direct part for near pairs,
// so only the spectral value is evaluated:
//   * k_near_sets: per near-source sphere, a sparse linear map (built on the host) takes the
//     sphere's vector-SH coefficients to coefficient sets of its exterior Laplace potentials
//     in irregular solid harmonics Th_n^m (degree <= p+3): 25 sets for the traction
//     (div L and the Hessians of L_x, L_y, L_z, L_r) or 15 for the single layer
//     (L_j, grad L_j, grad L_r);
//   * k_near_eval: one CTA per (target sphere, tile of its grid points) walks the target's
//     neighbour list in order, maps each point into the source's body frame scaled to the unit
//     sphere, evaluates Th_n^m column by column with the stable three-term recurrence and
//     contracts it with the sets (broadcast loads), then forms
//       4 pi t_i = n_i div L - x_j n_k d_i d_k L_j + n_k d_i d_k L_r       (traction)
//       8 pi u_i = L_i - x_j d_i L_j + d_i L_r                             (single layer, x radius)
//     and rotates back into the lab frame. Accumulation per target point is in a fixed order.
#include <atomic>

#include "df.h"
#include "smob_internal.h"
#include "tc_sm100.h"

namespace smob {

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

template <typename T>
__device__ __forceinline__ void qrot(const T* q, const T* v, T* o) {
    const T w = q[0], x = q[1], y = q[2], z = q[3];
    const T tx = 2 * (y * v[2] - z * v[1]);
    const T ty = 2 * (z * v[0] - x * v[2]);
    const T tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}

// Per near pair and target: the target in the source's body frame scaled to the unit sphere, and the
// target normal in the body frame. E is the arithmetic of this set-up and of the assembly below: FP32
// in the FP32 passes (the FP64 pipe of this GPU runs at 1/58 of the FP32 rate, and ~190 FP64 operations
// per pair cost more than the contraction itself), FP64 in the FP64 passes. The difference from the
// source centre is taken in FP64 either way (target and centre are large, their difference small).
template <typename E>
__device__ __forceinline__ void near_frame(const DevGeom& g, int s, const double* X, const E* nl, E* xs, E* nb) {
    const E q[4] = {E(g.quat[4 * s]), E(-g.quat[4 * s + 1]), E(-g.quat[4 * s + 2]), E(-g.quat[4 * s + 3])};
    const E rel[3] = {E(X[0] - g.center[3 * s]), E(X[1] - g.center[3 * s + 1]), E(X[2] - g.center[3 * s + 2])};
    E xb[3];
    qrot(q, rel, xb);
    qrot(q, nl, nb);
    const E a = E(g.radius[s]);
    if (sizeof(E) == 4) {
        const E ia = E(1) / a;
        for (int d = 0; d < 3; ++d) xs[d] = xb[d] * ia;
    } else {
        for (int d = 0; d < 3; ++d) xs[d] = xb[d] / a;
    }
}

// The traction (TRAC) or single-layer velocity at one target from its NS contracted sets, rotated back
// to the lab frame: 4 pi t_i = n_i div L - x_j n_k d_i d_k L_j + n_k d_i d_k L_r,
// 8 pi u_i = a (L_i - x_j d_i L_j + d_i L_r).
template <bool TRAC, typename E, typename A>
__device__ __forceinline__ void near_assemble(const DevGeom& g, int s, const A* acc, const E* xs, const E* nn,
                                              E* vl) {
    E vb[3];
    if (TRAC) {
        // symmetric index s(i,k): 00,11,22,01,02,12 -> 0..5
        const int S3[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
        for (int ii = 0; ii < 3; ++ii) {
            E v = nn[ii] * E(acc[0]);
            for (int kk = 0; kk < 3; ++kk) {
                E h = E(acc[19 + S3[ii][kk]]);
                for (int jj = 0; jj < 3; ++jj) h -= xs[jj] * E(acc[1 + 6 * jj + S3[ii][kk]]);
                v += nn[kk] * h;
            }
            vb[ii] = sizeof(E) == 4 ? v * E(1.0 / (4 * kPi)) : v / E(4 * kPi);
        }
    } else {
        const E a = E(g.radius[s]);
        for (int ii = 0; ii < 3; ++ii) {
            E v = E(acc[ii]) + E(acc[12 + ii]);
            for (int jj = 0; jj < 3; ++jj) v -= xs[jj] * E(acc[3 + 3 * jj + ii]);
            vb[ii] = sizeof(E) == 4 ? a * v * E(1.0 / (8 * kPi)) : a * v / E(8 * kPi);
        }
    }
    const E q[4] = {E(g.quat[4 * s]), E(g.quat[4 * s + 1]), E(g.quat[4 * s + 2]), E(g.quat[4 * s + 3])};
    qrot(q, vb, vl);
}

// Position of harmonic (n, m) in the recurrence order of degree Nd (m = 0..Nd outer, n = m..Nd inner),
// the K order of the tensor-core contraction.
__host__ __device__ __forceinline__ int rec_pos(int n, int m, int Nd) { return m * (Nd + 1) - m * (m - 1) / 2 + (n - m); }

// tiled = 2 (FP64 map): the [idx][set] complex layout with every value as a float pair (hi, lo) in the
// 8 bytes of the double, for the float-float kernel k_near_eval_df.
// tiled = 1: write the sets as the B operand of k_near_eval_tc instead of [idx][set] complex: per chunk of
// kNearTcChunk harmonics (in recurrence order) an NN x 2 kNearTcChunk FP32 tile in the K-major
// core-matrix layout of tc_sm100.h (row = set, K = (Re, -Im) of each harmonic); the padding (sets
// >= NS, harmonics past ncoef(p + 3)) stays as cleared at allocation.
template <typename Real>
__global__ void k_near_sets(DevGeom g, const Real* __restrict__ coef, const Real* __restrict__ mapval, bool trac,
                            const int* __restrict__ slot_sphere, long long stride, Real* __restrict__ sets,
                            int tiled) {
    const int slot = blockIdx.x;
    const int s = slot_sphere[slot];
    if (g.active && !g.active[g.prob[s]]) return;
    const int p = g.order[s];
    const OrderTables T = g.tabs[p];
    const int nc = T.nc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* cin = reinterpret_cast<Real*>(smem_raw);
    const Real* src = coef + 2LL * g.coff[s];
    for (int i = threadIdx.x; i < 6 * nc; i += blockDim.x) cin[i] = src[i];
    __syncthreads();
    const int base = trac ? T.trac_map : T.sl_map;
    const int rows = trac ? T.trac_rows : T.sl_rows;
    Real* out = sets + stride * slot;
    const int NS = trac ? kNearSetsTrac : kNearSetsSL;
    const int NN = trac ? 32 : 16;
    const int Nd = p + 3;
    for (int r = blockIdx.y * blockDim.x + threadIdx.x; r < rows; r += gridDim.y * blockDim.x) {
        const int e0 = g.map_rowptr[base + r], e1 = g.map_rowptr[base + r + 1];
        Real acc = 0;
        for (int e = e0; e < e1; ++e) acc += mapval[e] * cin[g.map_col[e]];
        if (!tiled) {
            out[r] = acc;
            continue;
        }
        if (tiled == 2) {
            // float-float sets for k_near_eval_df: the [idx][set] complex layout, each value (hi, lo)
            const float hi = float(acc);
            reinterpret_cast<float2*>(out)[r] = make_float2(hi, float(acc - double(hi)));
            continue;
        }
        // row r = (idx, set, re/im) of the [idx][set] complex layout
        const int idx = r / (2 * NS), rem = r - idx * 2 * NS, set = rem >> 1, im = rem & 1;
        int n = 0;
        while ((n + 1) * (n + 2) / 2 <= idx) ++n;
        const int pos = rec_pos(n, idx - n * (n + 1) / 2, Nd);
        const int ch = pos / kNearTcChunk, k = 2 * (pos - ch * kNearTcChunk) + im;
        out[(long long)ch * NN * (2 * kNearTcChunk) + tc::kmajor_offset(set, k, 2 * kNearTcChunk) / 4] = im ? -acc : acc;
    }
}

// (re, im) of one coefficient as one 8- or 16-byte load (the sets of a harmonic are (re, im) pairs)
template <typename Real>
struct Cplx;
template <>
struct Cplx<float> {
    using T = float2;
};
template <>
struct Cplx<double> {
    using T = double2;
};

// One target point per group of LANES lanes. Every lane runs the (cheap) harmonic recurrence;
// lane l contracts only the coefficient sets k = l, l + LANES, ..., so the lanes of a group read
// adjacent coefficients (one or two sectors per warp load, shared by the warp's groups) and the
// sets are gathered with shuffles for the final assembly. More lanes add parallelism for small
// problems at the price of repeating the recurrence; the host picks LANES from the number of
// target points that have near pairs.
// pair_filter: 0 every pair, 1 only pairs with gap >= 0.1 min radius, 2 only the
// near-singular pairs (gap < 0.1 min radius).
// PPT target points per thread share every coefficient load (one load, PPT complex multiply-adds).
// SMEM: the sets are staged in shared memory (plain loads) instead of read through the read-only cache.
template <typename Real, int NS, int LANES, int PPT, bool SMEM>
__device__ __forceinline__ void contract_lane(const Real* __restrict__ set, int idx, int lane, const Real* tr,
                                              const Real* ti, Real (*acc)[(NS + LANES - 1) / LANES]) {
    const typename Cplx<Real>::T* c = reinterpret_cast<const typename Cplx<Real>::T*>(set + 2 * NS * idx);
#pragma unroll
    for (int s = 0; s < (NS + LANES - 1) / LANES; ++s) {
        const int k = lane + LANES * s;
        if (k < NS) {
            const typename Cplx<Real>::T v = SMEM ? c[k] : __ldg(c + k);
#pragma unroll
            for (int p = 0; p < PPT; ++p) acc[p][s] = fma(v.x, tr[p], fma(-v.y, ti[p], acc[p][s]));
        }
    }
}

// Target points per thread: two in FP32 when one lane serves a target (many targets, e.g. batches),
// so each coefficient load feeds two points and the two recurrences run side by side; one otherwise
// (the FP64 variant would spill at the register budget that keeps 4 CTAs per SM).
template <typename Real, int LANES>
__host__ __device__ constexpr int near_ppt() { return (LANES == 1 && sizeof(Real) == 4) ? 2 : 1; }

// STAGE: each source's coefficient sets (NS x ncoef(p+3) complex values) and the recurrence tables are
// staged in dynamic shared memory, so the contraction reads shared memory instead of L1/L2; the
// arithmetic and its order are those of the unstaged kernel.
template <typename Real, bool TRAC, int LANES, bool STAGE>
// registers: two-point FP32 at 3 CTAs per SM (168 without spills), one-lane FP64 at 4 CTAs per SM
__global__ void __launch_bounds__(kNearThreads, near_ppt<Real, LANES>() == 2 ? 3 : (LANES == 1 ? 4 : 1))
    k_near_eval(DevGeom g, const Real* __restrict__ sets, long long stride, const Real* __restrict__ th, int th_c1,
                int th_c2, int th_diag, double c, int pair_filter, int tile_major, double* __restrict__ out) {
    constexpr int NS = TRAC ? kNearSetsTrac : kNearSetsSL;
    constexpr int kNearLanes = LANES;
    constexpr int PPT = near_ppt<Real, LANES>();
    constexpr int GROUPS = kNearThreads / kNearLanes;  // target groups per CTA and per point slot
    // tile-major grid: the tiles of one target sphere are adjacent in launch order, so they run
    // together and share its sources' coefficient sets through L2 instead of each fetching them
    const int t = tile_major ? blockIdx.y : blockIdx.x;
    const int tile = tile_major ? blockIdx.x : blockIdx.y;
    if (g.active && !g.active[g.prob[t]]) return;
    const int e0 = g.nbr_start[t], e1 = g.nbr_start[t + 1];
    if (e0 == e1) return;
    const int lane = threadIdx.x % kNearLanes;
    const int ng = g.glen[t];
    if (tile * GROUPS * PPT >= ng) return;  // whole CTA past the sphere
    bool valid[PPT];
    int i[PPT];
    double X[PPT][3], res[PPT][3];
    Real Nl[PPT][3];
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
        const int j = (tile * PPT + p) * GROUPS + threadIdx.x / kNearLanes;
        valid[p] = j < ng;  // lanes of an invalid point stay for the shuffles
        i[p] = g.gidx[t] + (valid[p] ? j : 0);
        for (int d = 0; d < 3; ++d) {
            X[p][d] = g.coords[3 * i[p] + d];
            Nl[p][d] = Real(g.norms[3 * i[p] + d]);
            res[p][d] = 0;
        }
    }
    const Real* c1 = th + th_c1;
    const Real* c2 = th + th_c2;
    const Real* dg = th + th_diag;
    // staged layout: [sets: 2 NS ncoef(pmax+3)][c1: ncoef][c2: ncoef][diag: pmax+4]
    extern __shared__ __align__(16) unsigned char near_smem[];
    Real* sS = reinterpret_cast<Real*>(near_smem);
    if (STAGE) {
        const int ncd = ncoef(g.pmax + 3);
        Real* t1 = sS + 2 * NS * ncd;
        for (int k = threadIdx.x; k < ncd; k += blockDim.x) {
            t1[k] = c1[k];
            t1[ncd + k] = c2[k];
        }
        for (int k = threadIdx.x; k < g.pmax + 4; k += blockDim.x) t1[2 * ncd + k] = dg[k];
        c1 = t1;
        c2 = t1 + ncd;
        dg = t1 + 2 * ncd;
    }
    for (int e = e0; e < e1; ++e) {
        if (pair_filter == 1 && g.nbr_precise[e]) continue;  // (uniform over the CTA)
        if (pair_filter == 2 && !g.nbr_precise[e]) continue;
        const int s = g.nbr_src[e];
        const int slot = g.near_src_slot[s];
        const Real* S = sets + stride * slot;
        const int Nd = g.order[s] + 3;
        if (STAGE) {
            // the previous source's sets are done; copy this source's, one complex value (8 or 16 bytes,
            // the slot stride's alignment) per load
            __syncthreads();
            using CT = typename Cplx<Real>::T;
            const int nv = NS * ncoef(Nd);
            const CT* srcv = reinterpret_cast<const CT*>(S);
            CT* dstv = reinterpret_cast<CT*>(sS);
            for (int k = threadIdx.x; k < nv; k += blockDim.x) dstv[k] = __ldg(srcv + k);
            __syncthreads();
            S = sS;
        }
        constexpr int NL = (NS + kNearLanes - 1) / kNearLanes;
        Real x[PPT], y[PPT], z[PPT], ir2[PPT], dr[PPT], di[PPT];
        Real nb[PPT][3];
        Real accl[PPT][NL];
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            Real xs[3];
            near_frame<Real>(g, s, X[p], Nl[p], xs, nb[p]);
            x[p] = xs[0];
            y[p] = xs[1];
            z[p] = xs[2];
            const Real r2 = x[p] * x[p] + y[p] * y[p] + z[p] * z[p];
            ir2[p] = Real(1) / r2;
            dr[p] = Real(1) / sqrt(r2);  // Th_0^0
            di[p] = 0;
#pragma unroll
            for (int k = 0; k < NL; ++k) accl[p][k] = 0;
        }
        for (int m = 0; m <= Nd; ++m) {
            Real pr[PPT], pi[PPT], cr[PPT], ci[PPT];
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                if (m > 0) {
                    const Real f = -dg[m] * ir2[p];
                    const Real nr = f * (x[p] * dr[p] - y[p] * di[p]);
                    const Real ni = f * (x[p] * di[p] + y[p] * dr[p]);
                    dr[p] = nr;
                    di[p] = ni;
                }
                pr[p] = 0;
                pi[p] = 0;
                cr[p] = dr[p];
                ci[p] = di[p];
            }
            for (int n = m; n <= Nd; ++n) {
                const int idx = n * (n + 1) / 2 + m;
                contract_lane<Real, NS, LANES, PPT, STAGE>(S, idx, lane, cr, ci, accl);
                if (n < Nd) {
                    const Real a1 = c1[idx], a2 = c2[idx];
#pragma unroll
                    for (int p = 0; p < PPT; ++p) {
                        const Real nr = -(a1 * z[p] * cr[p] + a2 * pr[p]) * ir2[p];
                        const Real ni = -(a1 * z[p] * ci[p] + a2 * pi[p]) * ir2[p];
                        pr[p] = cr[p];
                        pi[p] = ci[p];
                        cr[p] = nr;
                        ci[p] = ni;
                    }
                }
            }
        }
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            // gather the NS sets from their owning lanes (set k lives in lane k % kNearLanes, slot k / kNearLanes)
            Real acc[NS];
#pragma unroll
            for (int k = 0; k < NS; ++k)
                acc[k] = __shfl_sync(0xffffffffu, accl[p][k / kNearLanes], k % kNearLanes, kNearLanes);
            const Real xs[3] = {x[p], y[p], z[p]};
            Real vl[3];
            near_assemble<TRAC, Real, Real>(g, s, acc, xs, nb[p], vl);
            res[p][0] += double(vl[0]);
            res[p][1] += double(vl[1]);
            res[p][2] += double(vl[2]);
        }
    }
#pragma unroll
    for (int p = 0; p < PPT; ++p)
        if (valid[p] && lane == 0) {
            out[3 * i[p]] += c * res[p][0];
            out[3 * i[p] + 1] += c * res[p][1];
            out[3 * i[p] + 2] += c * res[p][2];
        }
}

// ---------------------------------------------------------------- float-float near field
// The near field of the high-precision passes (the mixed solve's residual pass, SMOB_PREC_FLOAT_FLOAT,
// the near-singular pairs of the FP32 passes) in float-float arithmetic on the FP32 pipes instead of
// FP64: GB300 runs FP64 at 1/58 of the FP32 rate, and the ~10^4 multiply-adds per target and source
// of the contraction dominate. The body frame (FP64 subtraction and rotation) and the assembly of the
// traction or velocity stay in FP64; the solid-harmonic recurrence and the contraction with the sets
// (float pairs written by k_near_sets) run in float-float (~2^-44 relative per operation, far below the
// 1e-10 the refinement residuals need). One target point per thread, the source's sets staged in shared
// memory when they fit, as in k_near_eval.
template <typename T>
__device__ __forceinline__ df1 dfd(T v) {  // FP64 value as a float pair
    const float h = float(v);
    return {h, float(double(v) - double(h))};
}
// Re(c Th) for complex c = (cr, ci) and Th = (tr, ti), unnormalised (as df_dot3)
__device__ __forceinline__ df1 df_cre(const float4& c, const df1& tr, const df1& ti) {
    const float p0 = v_mul(c.x, tr.h), p1 = v_mul(-c.z, ti.h);
    float lo = v_add(v_fma(c.x, tr.h, -p0), v_fma(-c.z, ti.h, -p1));
    lo = v_fma(c.x, tr.l, v_fma(c.y, tr.h, lo));
    lo = v_fma(-c.z, ti.l, v_fma(-c.w, ti.h, lo));
    const df1 s = two_sum(p0, p1);
    return {s.h, v_add(s.l, lo)};
}
__device__ __forceinline__ df1 df_neg(df1 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ df1 df_add(df1 a, df1 b) {
    const df1 s = two_sum(a.h, b.h);
    return {s.h, v_add(s.l, v_add(a.l, b.l))};
}

template <bool TRAC, bool STAGE>
__global__ void __launch_bounds__(kNearThreads, 2)
    k_near_eval_df(DevGeom g, const float2* __restrict__ sets, long long stride, const double* __restrict__ th,
                   int th_c1, int th_c2, int th_diag, double c, int pair_filter, int tile_major,
                   double* __restrict__ out) {
    constexpr int NS = TRAC ? kNearSetsTrac : kNearSetsSL;
    const int t = tile_major ? blockIdx.y : blockIdx.x;
    const int tile = tile_major ? blockIdx.x : blockIdx.y;
    if (g.active && !g.active[g.prob[t]]) return;
    const int e0 = g.nbr_start[t], e1 = g.nbr_start[t + 1];
    const int ng = g.glen[t];
    if (e0 == e1 || tile * kNearThreads >= ng) return;
    const int j = tile * kNearThreads + threadIdx.x;
    const bool valid = j < ng;
    const int i = g.gidx[t] + (valid ? j : 0);
    double X[3], Nl[3], res[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) {
        X[d] = g.coords[3 * i + d];
        Nl[d] = g.norms[3 * i + d];
    }
    // staged: [sets of one source: NS ncoef(pmax+3) complex as float4 (re hi, re lo, im hi, im lo)]
    // [c1, c2: ncoef(pmax+3) float pairs][diag: pmax+4 float pairs]
    extern __shared__ __align__(16) unsigned char near_df_smem[];
    const int ncd = ncoef(g.pmax + 3);
    float4* sS = reinterpret_cast<float4*>(near_df_smem);
    float4* t12 = sS + (STAGE ? NS * ncd : 0);  // (c1 hi, c1 lo, c2 hi, c2 lo)
    float2* tdg = reinterpret_cast<float2*>(t12 + ncd);
    for (int k = threadIdx.x; k < ncd; k += blockDim.x) {
        const df1 a = dfd(th[th_c1 + k]), b = dfd(th[th_c2 + k]);
        t12[k] = make_float4(a.h, a.l, b.h, b.l);
    }
    for (int k = threadIdx.x; k < g.pmax + 4; k += blockDim.x) {
        const df1 a = dfd(th[th_diag + k]);
        tdg[k] = make_float2(a.h, a.l);
    }
    __syncthreads();
    for (int e = e0; e < e1; ++e) {
        if (pair_filter == 1 && g.nbr_precise[e]) continue;  // (uniform over the CTA)
        if (pair_filter == 2 && !g.nbr_precise[e]) continue;
        const int s = g.nbr_src[e];
        const float4* S = reinterpret_cast<const float4*>(sets + stride * g.near_src_slot[s]);
        const int Nd = g.order[s] + 3;
        if (STAGE) {
            __syncthreads();  // the previous source's sets are done
            const int nv = NS * ncoef(Nd);
            for (int k = threadIdx.x; k < nv; k += blockDim.x) sS[k] = __ldg(S + k);
            __syncthreads();
            S = sS;
        }
        double xs[3], nb[3];
        near_frame<double>(g, s, X, Nl, xs, nb);
        const df1 x = dfd(xs[0]), y = dfd(xs[1]), z = dfd(xs[2]);
        const df1 r2 = df_sqr3(x, y, z);
        const df1 ri = df_rsqrt(r2);
        const df1 ir2 = df_mul_u(ri, ri);
        const df1 zi = df_mul_u(z, ir2);
        df1 dr = ri, di = {0.f, 0.f};  // Th_m^m
        df1 ah[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) ah[k] = {0.f, 0.f};
        for (int m = 0; m <= Nd; ++m) {
            if (m > 0) {
                // Th_m^m = -d_m (x + i y) Th_{m-1}^{m-1} / r^2
                const float2 dm = tdg[m];
                const df1 f = df_neg(df_mul_u(df1{dm.x, dm.y}, ir2));
                const df1 nr = df_mul_u(f, df_add(df_mul_u(x, dr), df_neg(df_mul_u(y, di))));
                const df1 ni = df_mul_u(f, df_add(df_mul_u(x, di), df_mul_u(y, dr)));
                dr = nr;
                di = ni;
            }
            df1 pr = {0.f, 0.f}, pi = {0.f, 0.f}, cr = dr, ci = di;
            for (int n = m; n <= Nd; ++n) {
                const int idx = n * (n + 1) / 2 + m;
                const float4* cs = S + NS * idx;
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    const df1 v = df_cre(cs[k], cr, ci);
                    df_acc(ah[k].h, ah[k].l, v);
                }
                if (n < Nd) {
                    // Th_{n+1}^m = -(c1 z Th_n^m + c2 Th_{n-1}^m) / r^2
                    const float4 a12 = t12[idx];
                    const df1 a1 = {a12.x, a12.y}, a2 = {a12.z, a12.w};
                    const df1 a1z = df_mul_u(a1, zi), a2r = df_mul_u(a2, ir2);
                    const df1 nr = df_neg(df_add(df_mul_u(a1z, cr), df_mul_u(a2r, pr)));
                    const df1 ni = df_neg(df_add(df_mul_u(a1z, ci), df_mul_u(a2r, pi)));
                    pr = cr;
                    pi = ci;
                    cr = nr;
                    ci = ni;
                }
            }
        }
        double acc[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) acc[k] = double(ah[k].h) + double(ah[k].l);
        double vl[3];
        near_assemble<TRAC, double, double>(g, s, acc, xs, nb, vl);
        res[0] += vl[0];
        res[1] += vl[1];
        res[2] += vl[2];
    }
    if (valid) {
        out[3 * i] += c * res[0];
        out[3 * i + 1] += c * res[1];
        out[3 * i + 2] += c * res[2];
    }
}

// ---------------------------------------------------------------- tensor-core near field (FP32 passes)
// The contraction of k_near_eval as a GEMM on the tcgen05 tensor cores. One CTA = 256 target points of
// one target sphere, one per thread, as two MMA tiles of M = 128 rows (threads 0-127, 128-255); for
// each near source sphere:
//   A [256 x K]: the targets' irregular solid harmonics, K = 2 ncoef(p_s + 3) real values (Re, Im of
//     each harmonic) in the recurrence order (m outer, n inner), generated by the threads
//     kNearTcChunk harmonics at a time (the FP32 recurrence of k_near_eval) into shared memory;
//   B [NN x K]: the source's coefficient sets as (Re, -Im) (tiled by k_near_sets), NN = 32 traction
//     (25 sets) or 16 single layer (15 sets), one chunk shared by both tiles;
//   D [128 x NN] per tile in tensor memory (tile 0 at column 0, tile 1 at column 32), FP32: row i holds
//     target i's NS contractions.
// Products in 3xTF32 (a_hi b_hi + a_hi b_lo + a_lo b_hi, the split made as the operands are staged).
// STAGES = 1: one operand stage per CTA (~72 KB, three CTAs per SM): the threads fill the chunk, one
// thread issues the MMAs, commits them to an mbarrier and waits for them (bounded) while the other warps
// sleep at the barrier and the other CTAs of the SM generate their chunks. STAGES = 2 (grids of about
// one CTA per SM, where no other CTA hides that wait): two stages and an mbarrier per stage; the thread
// that issues chunk k's MMAs then waits for chunk k - 1's, which ran while the threads generated chunk
// k, so the MMAs overlap the generation of the next chunk. The MMAs, their order and the accumulator
// are the same in both, so are the results. After a source's last chunk each warp loads its 32 rows
// (tcgen05.ld) and assembles the traction or velocity in FP32. On a wait timeout the CTA records it in
// err, writes nothing and releases its tensor memory.
constexpr int kTcK = 2 * kNearTcChunk;          // K per chunk (TF32 elements)
constexpr int kTcABytes = 128 * kTcK * 4;       // one A operand tile chunk (16 KB)
constexpr int kTcThreads = 256;                 // two M tiles
constexpr long long kTcWaitPolls = 1LL << 22;

template <bool TRAC>
__host__ __device__ constexpr int tc_nn() { return TRAC ? 32 : 16; }
// A hi, A lo for two tiles, then B hi, B lo
template <bool TRAC>
__host__ __device__ constexpr int tc_stage_bytes() { return 4 * kTcABytes + 2 * tc_nn<TRAC>() * kTcK * 4; }

template <bool TRAC, int STAGES>
__global__ void __launch_bounds__(kTcThreads, STAGES == 1 ? 2 : 1)
    k_near_eval_tc(DevGeom g, const float* __restrict__ tiles, long long tstride, const float* __restrict__ th,
                   int th_c1, int th_c2, int th_diag, double c, int pair_filter, int tile_major, double* __restrict__ out,
                   int* __restrict__ err) {
    constexpr int NS = TRAC ? kNearSetsTrac : kNearSetsSL;
    constexpr int NN = tc_nn<TRAC>();
    constexpr int BBYTES = NN * kTcK * 4;
    const int t = tile_major ? blockIdx.y : blockIdx.x;
    const int tile = tile_major ? blockIdx.x : blockIdx.y;
    if (g.active && !g.active[g.prob[t]]) return;
    const int e0 = g.nbr_start[t], e1 = g.nbr_start[t + 1];
    const int ng = g.glen[t];
    if (e0 == e1 || tile * kTcThreads >= ng) return;
    bool any = false;  // (uniform over the CTA)
    for (int e = e0; e < e1; ++e)
        if (!(pair_filter == 1 && g.nbr_precise[e]) && !(pair_filter == 2 && !g.nbr_precise[e])) any = true;
    if (!any) return;

    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ uint64_t mbar[STAGES];
    __shared__ uint32_t tbase;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, mt = tid >> 7, row = tid & 127;
    // recurrence tables after the stages: (c1, c2) pairs, then the diagonal factors
    const int ncd = ncoef(g.pmax + 3);
    float2* t12 = reinterpret_cast<float2*>(tc_smem + STAGES * tc_stage_bytes<TRAC>());
    float* dg = reinterpret_cast<float*>(t12 + ncd);
    for (int k = tid; k < ncd; k += kTcThreads) t12[k] = make_float2(th[th_c1 + k], th[th_c2 + k]);
    for (int k = tid; k < g.pmax + 4; k += kTcThreads) dg[k] = th[th_diag + k];
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < STAGES; ++q) tc::mbar_init(&mbar[q], 1);
        tc::mbar_fence_init();
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    constexpr uint32_t idesc = tc::idesc_tf32(128, NN);

    const int j = tile * kTcThreads + tid;
    const bool valid = j < ng;
    const int i = g.gidx[t] + (valid ? j : 0);
    double X[3], res[3] = {0, 0, 0};
    float Nl[3];
    for (int d = 0; d < 3; ++d) {
        X[d] = g.coords[3 * i + d];
        Nl[d] = float(g.norms[3 * i + d]);
    }
    unsigned phases = 0;  // bit q: the parity the next wait on mbar[q] expects
    bool failed = false;
    for (int e = e0; e < e1 && !failed; ++e) {
        if (pair_filter == 1 && g.nbr_precise[e]) continue;
        if (pair_filter == 2 && !g.nbr_precise[e]) continue;
        const int s = g.nbr_src[e];
        const float* T = tiles + tstride * g.near_src_slot[s];
        const int Nd = g.order[s] + 3;
        const int nck = (ncoef(Nd) + kNearTcChunk - 1) / kNearTcChunk;
        float xs3[3], nb[3];
        near_frame<float>(g, s, X, Nl, xs3, nb);
        const float x = xs3[0], y = xs3[1], z = xs3[2];
        const float r2 = x * x + y * y + z * z;
        const float ir2 = 1.f / r2;
        // recurrence state: the harmonic (n, m) to emit next is (cr, ci); past the last one (m > Nd) all zero
        float dr = 1.f / sqrtf(r2), di = 0.f;  // Th_m^m
        int m = 0, n = 0, idx = 0;              // idx = n (n + 1) / 2 + m
        float pr = 0.f, pi = 0.f, cr = dr, ci = di;
        const float zi = z * ir2;
        for (int ch = 0; ch < nck; ++ch) {
            const int stg = STAGES == 2 ? (ch & 1) : 0;
            unsigned char* const stage = tc_smem + stg * tc_stage_bytes<TRAC>();
            unsigned char* sA = stage + mt * 2 * kTcABytes;  // this thread's tile: hi, then lo
            unsigned char* sB = stage + 4 * kTcABytes;       // hi, then lo
            // B chunk (at most one float4 per thread): its load is issued first and lands while the
            // thread generates its A chunk; split and stored after that
            constexpr int kBVec = NN * kTcK / 4;
            static_assert(kBVec <= kTcThreads, "one B float4 per thread at most");
            const float4* gB = reinterpret_cast<const float4*>(T + (long long)ch * NN * kTcK);
            float4 bpre = make_float4(0.f, 0.f, 0.f, 0.f);
            if (tid < kBVec) bpre = __ldg(gB + tid);
            // A chunk: the next kNearTcChunk harmonics of this thread's target, 4 K values at a time
#pragma unroll
            for (int qd = 0; qd < kTcK / 4; ++qd) {
                float v4[4];
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    v4[2 * h2] = cr;
                    v4[2 * h2 + 1] = ci;
                    if (n < Nd) {
                        // Th_{n+1}^m = -(c1 z Th_n^m + c2 Th_{n-1}^m) / r^2
                        const float2 a12 = t12[idx];
                        const float nr = -(a12.x * zi * cr + a12.y * ir2 * pr);
                        const float ni = -(a12.x * zi * ci + a12.y * ir2 * pi);
                        pr = cr;
                        pi = ci;
                        cr = nr;
                        ci = ni;
                        idx += n + 1;
                        ++n;
                    } else if (m < Nd) {
                        // next column: Th_{m+1}^{m+1} = -d_{m+1} (x + i y) Th_m^m / r^2
                        ++m;
                        const float f = -dg[m] * ir2;
                        const float nr = f * (x * dr - y * di);
                        const float ni = f * (x * di + y * dr);
                        dr = nr;
                        di = ni;
                        pr = 0.f;
                        pi = 0.f;
                        cr = dr;
                        ci = di;
                        n = m;
                        idx = m * (m + 1) / 2 + m;
                    } else {
                        cr = 0.f;
                        ci = 0.f;
                    }
                }
                float4 h, l;
                tc::tf32_split(v4[0], h.x, l.x);
                tc::tf32_split(v4[1], h.y, l.y);
                tc::tf32_split(v4[2], h.z, l.z);
                tc::tf32_split(v4[3], h.w, l.w);
                const uint32_t off = tc::kmajor_offset(row, 4 * qd, kTcK);
                *reinterpret_cast<float4*>(sA + off) = h;
                *reinterpret_cast<float4*>(sA + kTcABytes + off) = l;
            }
            if (tid < kBVec) {
                float4 h, l;
                tc::tf32_split(bpre.x, h.x, l.x);
                tc::tf32_split(bpre.y, h.y, l.y);
                tc::tf32_split(bpre.z, h.z, l.z);
                tc::tf32_split(bpre.w, h.w, l.w);
                reinterpret_cast<float4*>(sB)[tid] = h;
                reinterpret_cast<float4*>(sB + BBYTES)[tid] = l;
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t b0 = tc::smem_u32(sB), bl0 = b0 + BBYTES;
#pragma unroll
                for (int tt = 0; tt < 2; ++tt) {
                    const uint32_t a0 = tc::smem_u32(stage + tt * 2 * kTcABytes), al0 = a0 + kTcABytes;
#pragma unroll
                    for (int ks = 0; ks < kTcK / 8; ++ks) {
                        const uint32_t o = ks * 256;
                        const uint64_t ah = tc::sdesc(a0 + o, 128, (kTcK / 4) * 128);
                        const uint64_t al = tc::sdesc(al0 + o, 128, (kTcK / 4) * 128);
                        const uint64_t bh = tc::sdesc(b0 + o, 128, (kTcK / 4) * 128);
                        const uint64_t bl = tc::sdesc(bl0 + o, 128, (kTcK / 4) * 128);
                        const uint32_t d = tmem + 32 * tt;
                        tc::mma_tf32(d, ah, bh, idesc, ch > 0 || ks > 0);
                        tc::mma_tf32(d, ah, bl, idesc, true);
                        tc::mma_tf32(d, al, bh, idesc, true);
                    }
                }
                tc::mma_commit(&mbar[stg]);
                // one thread waits (the others sleep at the barrier below): for this chunk's MMAs with
                // one stage, for the previous chunk's with two (its stage is filled next)
                if (STAGES == 1) {
                    if (!tc::mbar_wait_bounded(&mbar[0], phases & 1u, kTcWaitPolls)) s_fail = 1;
                } else if (ch > 0) {
                    if (!tc::mbar_wait_bounded(&mbar[stg ^ 1], (phases >> (stg ^ 1)) & 1u, kTcWaitPolls)) s_fail = 1;
                }
            }
            if (STAGES == 1) phases ^= 1u;
            else if (ch > 0) phases ^= 1u << (stg ^ 1);
            __syncthreads();
            if (s_fail) {
                failed = true;
                break;
            }
        }
        if (failed) break;
        if (STAGES == 2) {  // the source's last chunk
            const int lst = (nck - 1) & 1;
            if (tid == 0 && !tc::mbar_wait_bounded(&mbar[lst], (phases >> lst) & 1u, kTcWaitPolls)) s_fail = 1;
            phases ^= 1u << lst;
            __syncthreads();
            if (s_fail) {
                failed = true;
                break;
            }
        }
        tc::fence_after_sync();
        float acc[32];
        tc::tmem_ld_32x32b_x32(tmem + 32 * mt + (uint32_t((warp & 3) * 32) << 16), acc);
        tc::fence_before_sync();  // the next source's first MMA overwrites D after the next barrier
        (void)NS;
        float vl[3];
        near_assemble<TRAC, float, float>(g, s, acc, xs3, nb, vl);
        res[0] += double(vl[0]);
        res[1] += double(vl[1]);
        res[2] += double(vl[2]);
    }
    if (failed) {
        if (tid == 0) atomicExch(err, 1);
    } else if (valid) {
        out[3 * i] += c * res[0];
        out[3 * i + 1] += c * res[1];
        out[3 * i + 2] += c * res[2];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 64);
    }
}

}  // namespace

int launch_near_sets(const DevGeom& g, const void* coef, bool trac, bool fp32, void* sets, int nslots,
                     const int* slot_sphere, long long stride, cudaStream_t st, bool df) {
    if (nslots <= 0) return 0;
    const size_t sm = size_t(6 * ncoef(g.pmax)) * (fp32 ? sizeof(float) : sizeof(double));
    // each slot's rows (2 x sets x ncoef(p+3), ~10^4) split over CTAs: few near-source spheres still give
    // the GPU enough CTAs. Each row is one thread's fixed sum, so the split leaves every value unchanged;
    // 32 for at most 64 slots (cfg2: the sets 0.39 instead of 0.50 ms per solve, 97.0 against 96.7
    // solves/s), else 8, where each CTA's copy of the coefficients would cost more than the finer split
    const int split = nslots <= 64 ? 32 : 8;
    const dim3 grid(nslots, split);
    if (fp32) {
        const bool tiled = g.near_tc != 0;
        k_near_sets<float><<<grid, 256, sm, st>>>(g, static_cast<const float*>(coef), g.map_val_f, trac, slot_sphere,
                                                  tiled ? near_tile_stride(g.pmax, trac) : stride,
                                                  static_cast<float*>(sets), tiled ? 1 : 0);
    } else {
        k_near_sets<double><<<grid, 256, sm, st>>>(g, static_cast<const double*>(coef), g.map_val_d, trac,
                                                   slot_sphere, stride, static_cast<double*>(sets), df ? 2 : 0);
    }
    return 1;
}

// dynamic shared memory of the staged near kernel: sets of one source, c1, c2, diag
template <typename Real>
size_t near_stage_bytes(int pmax, bool trac) {
    const size_t ncd = ncoef(pmax + 3);
    return (2 * (trac ? kNearSetsTrac : kNearSetsSL) * ncd + 2 * ncd + pmax + 4) * sizeof(Real);
}
constexpr size_t kNearStageMax = 160 * 1024;  // larger set blocks (FP64 at high orders) read through L1/L2

template <typename Real, bool TRAC, int LANES>
void launch_near_typed(const DevGeom& g, dim3 grid, const Real* s, const Real* tab, long long stride, double c,
                       int pair_filter, int tm, double* out, cudaStream_t st) {
    const size_t sm = near_stage_bytes<Real>(g.pmax, TRAC);
    if (sm <= kNearStageMax)
        k_near_eval<Real, TRAC, LANES, true><<<grid, kNearThreads, sm, st>>>(g, s, stride, tab, g.th_c1, g.th_c2,
                                                                            g.th_diag, c, pair_filter, tm, out);
    else
        k_near_eval<Real, TRAC, LANES, false><<<grid, kNearThreads, 0, st>>>(g, s, stride, tab, g.th_c1, g.th_c2,
                                                                            g.th_diag, c, pair_filter, tm, out);
}

template <int LANES>
void launch_near_eval_l(const DevGeom& g, const void* sets, long long stride, bool trac, bool fp32, double c,
                        double* out, cudaStream_t st, int pair_filter) {
    const int gmax = (g.pmax + 1) * (2 * g.pmax + 2);
    const int per_cta = kNearThreads / LANES * (fp32 ? near_ppt<float, LANES>() : 1);
    const int tiles = (gmax + per_cta - 1) / per_cta;
    const int tm = g.N <= 65535 ? 1 : 0;  // grid y is limited to 65535
    const dim3 grid = tm ? dim3(tiles, g.N) : dim3(g.N, tiles);
    if (fp32) {
        const float* s = static_cast<const float*>(sets);
        if (trac) launch_near_typed<float, true, LANES>(g, grid, s, g.tab_f, stride, c, pair_filter, tm, out, st);
        else launch_near_typed<float, false, LANES>(g, grid, s, g.tab_f, stride, c, pair_filter, tm, out, st);
    } else {
        const double* s = static_cast<const double*>(sets);
        if (trac) launch_near_typed<double, true, LANES>(g, grid, s, g.tab_d, stride, c, pair_filter, tm, out, st);
        else launch_near_typed<double, false, LANES>(g, grid, s, g.tab_d, stride, c, pair_filter, tm, out, st);
    }
}

template <typename Real, bool TRAC>
void configure_near_typed() {
    cudaFuncSetAttribute(k_near_eval<Real, TRAC, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
    cudaFuncSetAttribute(k_near_eval<Real, TRAC, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
    cudaFuncSetAttribute(k_near_eval<Real, TRAC, 4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
    cudaFuncSetAttribute(k_near_eval<Real, TRAC, 8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
}

// dynamic shared memory of the float-float near kernel: one source's sets (staged) and the tables
template <bool TRAC>
size_t near_df_smem(int pmax, bool stage) {
    const size_t ncd = ncoef(pmax + 3);
    return (stage ? size_t(TRAC ? kNearSetsTrac : kNearSetsSL) * ncd * 16 : 0) + ncd * 16 + size_t(pmax + 4) * 8;
}

// dynamic shared memory of the tensor-core near kernel: the operand stages and the recurrence tables
template <bool TRAC>
size_t near_tc_smem(int pmax, int stages) {
    return size_t(stages) * size_t(tc_stage_bytes<TRAC>()) + size_t(2 * ncoef(pmax + 3) + pmax + 4) * sizeof(float);
}

void configure_near_kernels() {
    cudaFuncSetAttribute(k_near_eval_df<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
    cudaFuncSetAttribute(k_near_eval_df<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNearStageMax));
    cudaFuncSetAttribute(k_near_eval_df<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_df_smem<true>(kMaxOrder, false)));
    cudaFuncSetAttribute(k_near_eval_df<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_df_smem<false>(kMaxOrder, false)));
    cudaFuncSetAttribute(k_near_eval_tc<true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_tc_smem<true>(kMaxOrder, 1)));
    cudaFuncSetAttribute(k_near_eval_tc<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_tc_smem<false>(kMaxOrder, 1)));
    cudaFuncSetAttribute(k_near_eval_tc<true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_tc_smem<true>(kMaxOrder, 2)));
    cudaFuncSetAttribute(k_near_eval_tc<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(near_tc_smem<false>(kMaxOrder, 2)));
    configure_near_typed<float, true>();
    configure_near_typed<float, false>();
    configure_near_typed<double, true>();
    configure_near_typed<double, false>();
}

template <bool TRAC>
void launch_near_df_typed(const DevGeom& g, const void* sets, long long stride, double c, int pair_filter,
                          double* out, cudaStream_t st) {
    const int gmax = (g.pmax + 1) * (2 * g.pmax + 2);
    const int tiles = (gmax + kNearThreads - 1) / kNearThreads;
    const int tm = g.N <= 65535 ? 1 : 0;
    const dim3 grid = tm ? dim3(tiles, g.N) : dim3(g.N, tiles);
    const float2* sp = static_cast<const float2*>(sets);
    const size_t sm = near_df_smem<TRAC>(g.pmax, true);
    if (sm <= kNearStageMax)
        k_near_eval_df<TRAC, true><<<grid, kNearThreads, sm, st>>>(g, sp, stride, g.tab_d, g.th_c1, g.th_c2,
                                                                   g.th_diag, c, pair_filter, tm, out);
    else
        k_near_eval_df<TRAC, false><<<grid, kNearThreads, near_df_smem<TRAC>(g.pmax, false), st>>>(
            g, sp, stride, g.tab_d, g.th_c1, g.th_c2, g.th_diag, c, pair_filter, tm, out);
}

// SMs of the current device, looked up once per device
static int sm_count() {
    constexpr int kDevices = 64;
    static std::atomic<int> cache[kDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    int v = dev >= 0 && dev < kDevices ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (v == 0) {
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (dev >= 0 && dev < kDevices) cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

int launch_near_eval(const DevGeom& g, const void* sets, long long stride, bool trac, bool fp32, double c, double* out,
                     cudaStream_t st, int pair_filter, bool df) {
    if (df && !fp32) {
        if (trac) launch_near_df_typed<true>(g, sets, stride, c, pair_filter, out, st);
        else launch_near_df_typed<false>(g, sets, stride, c, pair_filter, out, st);
        return 1;
    }
    if (fp32 && g.near_tc) {
        // one CTA per (target sphere, 256 of its grid points); tile-major (the tiles of a sphere adjacent)
        const int gmax = (g.pmax + 1) * (2 * g.pmax + 2);
        const int tiles = (gmax + kTcThreads - 1) / kTcThreads;
        const int tm = g.N <= 65535 ? 1 : 0;
        const dim3 grid = tm ? dim3(tiles, g.N) : dim3(g.N, tiles);
        const float* tl = static_cast<const float*>(sets);
        // two operand stages when the grid is about one wave of one CTA per SM (the same results)
        const bool two = (long long)grid.x * grid.y <= 2LL * sm_count();
        const long long tsv = near_tile_stride(g.pmax, trac);
        if (trac && two)
            k_near_eval_tc<true, 2><<<grid, kTcThreads, near_tc_smem<true>(g.pmax, 2), st>>>(
                g, tl, tsv, g.tab_f, g.th_c1, g.th_c2, g.th_diag, c, pair_filter, tm, out, g.err);
        else if (trac)
            k_near_eval_tc<true, 1><<<grid, kTcThreads, near_tc_smem<true>(g.pmax, 1), st>>>(
                g, tl, tsv, g.tab_f, g.th_c1, g.th_c2, g.th_diag, c, pair_filter, tm, out, g.err);
        else if (two)
            k_near_eval_tc<false, 2><<<grid, kTcThreads, near_tc_smem<false>(g.pmax, 2), st>>>(
                g, tl, tsv, g.tab_f, g.th_c1, g.th_c2, g.th_diag, c, pair_filter, tm, out, g.err);
        else
            k_near_eval_tc<false, 1><<<grid, kTcThreads, near_tc_smem<false>(g.pmax, 1), st>>>(
                g, tl, tsv, g.tab_f, g.th_c1, g.th_c2, g.th_diag, c, pair_filter, tm, out, g.err);
        return 1;
    }
    switch (g.near_lanes) {
        case 1: launch_near_eval_l<1>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        case 2: launch_near_eval_l<2>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        case 4: launch_near_eval_l<4>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        default: launch_near_eval_l<8>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
    }
    return 1;
}

}  // namespace smob
