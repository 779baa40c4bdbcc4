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
#include "smob_internal.h"

namespace smob {

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

__device__ __forceinline__ void qrot(const double* q, const double* v, double* o) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double tx = 2 * (y * v[2] - z * v[1]);
    const double ty = 2 * (z * v[0] - x * v[2]);
    const double tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}

template <typename Real>
__global__ void k_near_sets(DevGeom g, const Real* __restrict__ coef, const Real* __restrict__ mapval, bool trac,
                            const int* __restrict__ slot_sphere, long long stride, Real* __restrict__ sets) {
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
    for (int r = blockIdx.y * blockDim.x + threadIdx.x; r < rows; r += gridDim.y * blockDim.x) {
        const int e0 = g.map_rowptr[base + r], e1 = g.map_rowptr[base + r + 1];
        Real acc = 0;
        for (int e = e0; e < e1; ++e) acc += mapval[e] * cin[g.map_col[e]];
        out[r] = acc;
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
    double X[PPT][3], Nl[PPT][3], res[PPT][3];
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
        const int j = (tile * PPT + p) * GROUPS + threadIdx.x / kNearLanes;
        valid[p] = j < ng;  // lanes of an invalid point stay for the shuffles
        i[p] = g.gidx[t] + (valid[p] ? j : 0);
        for (int d = 0; d < 3; ++d) {
            X[p][d] = g.coords[3 * i[p] + d];
            Nl[p][d] = g.norms[3 * i[p] + d];
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
        const double q[4] = {g.quat[4 * s], g.quat[4 * s + 1], g.quat[4 * s + 2], g.quat[4 * s + 3]};
        const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
        const double a = g.radius[s];
        constexpr int NL = (NS + kNearLanes - 1) / kNearLanes;
        Real x[PPT], y[PPT], z[PPT], ir2[PPT], dr[PPT], di[PPT];
        double nb[PPT][3];
        Real accl[PPT][NL];
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            const double rel[3] = {X[p][0] - g.center[3 * s], X[p][1] - g.center[3 * s + 1],
                                   X[p][2] - g.center[3 * s + 2]};
            double xb[3];
            qrot(qc, rel, xb);
            qrot(qc, Nl[p], nb[p]);
            x[p] = Real(xb[0] / a);
            y[p] = Real(xb[1] / a);
            z[p] = Real(xb[2] / a);
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
            double vb[3];
            const double xs[3] = {double(x[p]), double(y[p]), double(z[p])};
            if (TRAC) {
                // symmetric index s(i,k): 00,11,22,01,02,12 -> 0..5
                const int S3[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
                const double* nn = nb[p];
                for (int ii = 0; ii < 3; ++ii) {
                    double v = nn[ii] * double(acc[0]);
                    for (int kk = 0; kk < 3; ++kk) {
                        double h = double(acc[19 + S3[ii][kk]]);
                        for (int jj = 0; jj < 3; ++jj) h -= xs[jj] * double(acc[1 + 6 * jj + S3[ii][kk]]);
                        v += nn[kk] * h;
                    }
                    vb[ii] = v / (4 * kPi);
                }
            } else {
                for (int ii = 0; ii < 3; ++ii) {
                    double v = double(acc[ii]) + double(acc[12 + ii]);
                    for (int jj = 0; jj < 3; ++jj) v -= xs[jj] * double(acc[3 + 3 * jj + ii]);
                    vb[ii] = a * v / (8 * kPi);
                }
            }
            double vl[3];
            qrot(q, vb, vl);
            res[p][0] += vl[0];
            res[p][1] += vl[1];
            res[p][2] += vl[2];
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

}  // namespace

int launch_near_sets(const DevGeom& g, const void* coef, bool trac, bool fp32, void* sets, int nslots,
                     const int* slot_sphere, long long stride, cudaStream_t st) {
    if (nslots <= 0) return 0;
    const size_t sm = size_t(6 * ncoef(g.pmax)) * (fp32 ? sizeof(float) : sizeof(double));
    // each slot's rows (2 x sets x ncoef(p+3), ~10^4) split over kSetSplit CTAs: few near-source spheres
    // still give the GPU enough CTAs
    constexpr int kSetSplit = 8;
    const dim3 grid(nslots, kSetSplit);
    if (fp32)
        k_near_sets<float><<<grid, 256, sm, st>>>(g, static_cast<const float*>(coef), g.map_val_f, trac, slot_sphere,
                                                  stride, static_cast<float*>(sets));
    else
        k_near_sets<double><<<grid, 256, sm, st>>>(g, static_cast<const double*>(coef), g.map_val_d, trac,
                                                   slot_sphere, stride, static_cast<double*>(sets));
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

void configure_near_kernels() {
    configure_near_typed<float, true>();
    configure_near_typed<float, false>();
    configure_near_typed<double, true>();
    configure_near_typed<double, false>();
}

int launch_near_eval(const DevGeom& g, const void* sets, long long stride, bool trac, bool fp32, double c, double* out,
                     cudaStream_t st, int pair_filter) {
    switch (g.near_lanes) {
        case 1: launch_near_eval_l<1>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        case 2: launch_near_eval_l<2>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        case 4: launch_near_eval_l<4>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
        default: launch_near_eval_l<8>(g, sets, stride, trac, fp32, c, out, st, pair_filter); break;
    }
    return 1;
}

}  // namespace smob
