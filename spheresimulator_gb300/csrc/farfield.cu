// farfield.cu — all-pairs Stokes single-layer / traction far field.
//
// Replaces the STKFMM far-field evaluations of BIE/SphereSTKSHOperator.cpp:273-303 (PVel)
// and :354-446 (Traction, dotted with the target normal) by direct summation:
//   SL:        u(x) = 1/(8 pi) sum_y [ f/r + (r.f) r / r^3 ]
//   traction:  t(x) = -3/(4 pi) sum_y r (r.f)(r.n_x) / r^5,      r = x - y, f = w_y * density_y * c
// Sources on the target's own sphere are skipped (the reference adds then subtracts them,
// :306-351 and :375-433) and so are sources on the target's near-pair spheres (the
// reference subtracts their direct sum and adds the spectral value, :575-695); both are
// accounted for spectrally by the sphere and near kernels, so the sum here is exactly the
// remaining smooth-quadrature part.
//
// Work decomposition: one CTA per work item = (block of targets of one problem) x (chunk of
// source spheres of the same problem). Sources are staged per sphere in shared memory as
// float4 (x,y,z,sphere-id) + float4 (f,0); each thread owns two targets (FP32) or one (FP64).
// A per-thread merge cursor over the sorted near-pair list decides per source sphere whether
// the thread's target skips it; a CTA-wide vote skips the staging when every target does.
// Partial sums go to [problem][chunk][point][3] and a second kernel reduces the chunks in
// fixed order, so results do not depend on scheduling or on other problems in the batch.
#include "smob_internal.h"

namespace smob {

namespace {

__device__ __forceinline__ void pair_trac32(const float4& t, const float4& n, const float4& s, const float4& f,
                                            float& ax, float& ay, float& az) {
    const float rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float ri = rsqrtf(r2);
    const float ri2 = ri * ri;
    const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
    const float rn = fmaf(rx, n.x, fmaf(ry, n.y, rz * n.z));
    const float k = (rf * rn) * (ri2 * ri2 * ri);
    ax = fmaf(k, rx, ax);
    ay = fmaf(k, ry, ay);
    az = fmaf(k, rz, az);
}

__device__ __forceinline__ void pair_sl32(const float4& t, const float4& s, const float4& f, float& ax, float& ay,
                                          float& az) {
    const float rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float ri = rsqrtf(r2);
    const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
    const float k = rf * ri * ri * ri;
    ax = fmaf(f.x, ri, fmaf(k, rx, ax));
    ay = fmaf(f.y, ri, fmaf(k, ry, ay));
    az = fmaf(f.z, ri, fmaf(k, rz, az));
}

__device__ __forceinline__ void pair_trac64(const double4& t, const double4& n, const double4& s, const double4& f,
                                            double& ax, double& ay, double& az) {
    const double rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
    const double ri = rsqrt(r2);
    const double ri2 = ri * ri;
    const double rf = fma(rx, f.x, fma(ry, f.y, rz * f.z));
    const double rn = fma(rx, n.x, fma(ry, n.y, rz * n.z));
    const double k = (rf * rn) * (ri2 * ri2 * ri);
    ax = fma(k, rx, ax);
    ay = fma(k, ry, ay);
    az = fma(k, rz, az);
}

__device__ __forceinline__ void pair_sl64(const double4& t, const double4& s, const double4& f, double& ax,
                                          double& ay, double& az) {
    const double rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
    const double ri = rsqrt(r2);
    const double rf = fma(rx, f.x, fma(ry, f.y, rz * f.z));
    const double k = rf * ri * ri * ri;
    ax = fma(f.x, ri, fma(k, rx, ax));
    ay = fma(f.y, ri, fma(k, ry, ay));
    az = fma(f.z, ri, fma(k, rz, az));
}

// advance a thread's cursor over its target sphere's sorted near-source list; true if s is excluded
__device__ __forceinline__ bool excluded(const int* __restrict__ nbr_src, int& cur, int end, int sid, int s) {
    if (s == sid) return true;
    while (cur < end && __ldg(nbr_src + cur) < s) ++cur;
    return cur < end && __ldg(nbr_src + cur) == s;
}

// TPT targets per thread (register blocking: each staged source serves TPT pairs); a work item
// covers kFarThreads * TPT targets. The tile holds kFarTile32 sources, enough for a whole p=16
// sphere, so most source spheres cost one staging round and two barriers.
template <bool TRAC, int TPT>
__global__ void __launch_bounds__(kFarThreads) k_far32(DevGeom g, const FarItem* __restrict__ items,
                                                      const float4* __restrict__ src, float* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ float4 sp[kFarTile32];
    __shared__ float4 sf[kFarTile32];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 P[TPT], Nn[TPT];
    int sid[TPT], cur[TPT], end[TPT];
    bool val[TPT];
    float ax[TPT], ay[TPT], az[TPT];
#pragma unroll
    for (int u = 0; u < TPT; ++u) {
        const int t = it.t0 + threadIdx.x + u * kFarThreads;
        val[u] = t < it.t1;
        P[u] = val[u] ? g.pos32[t] : z4;
        Nn[u] = (TRAC && val[u]) ? g.nrm32[t] : z4;
        sid[u] = val[u] ? __float_as_int(P[u].w) : -1;
        cur[u] = val[u] ? g.nbr_start[sid[u]] : 0;
        end[u] = val[u] ? g.nbr_start[sid[u] + 1] : 0;
        ax[u] = ay[u] = az[u] = 0.f;
    }
    for (int s = it.s0; s < it.s1; ++s) {
        bool sk[TPT];
        bool all = true, none = true;
#pragma unroll
        for (int u = 0; u < TPT; ++u) {
            sk[u] = !val[u] || excluded(g.nbr_src, cur[u], end[u], sid[u], s);
            all = all && sk[u];
            none = none && !sk[u];
        }
        if (__syncthreads_and(all)) continue;
        const int g0 = g.gidx[s], gl = g.glen[s];
        for (int base = 0; base < gl; base += kFarTile32) {
            const int n = min(kFarTile32, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sp[k] = g.pos32[g0 + base + k];
                sf[k] = src[g0 + base + k];
            }
            __syncthreads();
            if (none) {
#pragma unroll 4
                for (int k = 0; k < n; ++k) {
                    const float4 q = sp[k], f = sf[k];
#pragma unroll
                    for (int u = 0; u < TPT; ++u) {
                        if (TRAC) pair_trac32(P[u], Nn[u], q, f, ax[u], ay[u], az[u]);
                        else pair_sl32(P[u], q, f, ax[u], ay[u], az[u]);
                    }
                }
            } else {
                for (int k = 0; k < n; ++k) {
                    const float4 q = sp[k], f = sf[k];
#pragma unroll
                    for (int u = 0; u < TPT; ++u) {
                        if (sk[u]) continue;
                        if (TRAC) pair_trac32(P[u], Nn[u], q, f, ax[u], ay[u], az[u]);
                        else pair_sl32(P[u], q, f, ax[u], ay[u], az[u]);
                    }
                }
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
    float* out = partial + pr.poff + 3LL * mp * it.chunk;
#pragma unroll
    for (int u = 0; u < TPT; ++u) {
        if (!val[u]) continue;
        float* o = out + 3LL * (it.t0 + threadIdx.x + u * kFarThreads - pr.p0);
        o[0] = ax[u];
        o[1] = ay[u];
        o[2] = az[u];
    }
}

template <bool TRAC>
__global__ void __launch_bounds__(kFarThreads) k_far64(DevGeom g, const FarItem* __restrict__ items,
                                                      const double4* __restrict__ src, double* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ double4 sp[kFarTile];
    __shared__ double4 sf[kFarTile];
    const int ta = it.t0 + threadIdx.x;
    const bool va = ta < it.t1;
    const double4 z4 = make_double4(0, 0, 0, 0);
    const double4 pa = va ? g.pos64[ta] : z4;
    const double4 na = (TRAC && va) ? g.nrm64[ta] : z4;
    const int sa = va ? g.sid[ta] : -1;
    int ca = va ? g.nbr_start[sa] : 0, ea = va ? g.nbr_start[sa + 1] : 0;
    double xa = 0, ya = 0, za = 0;
    for (int s = it.s0; s < it.s1; ++s) {
        const bool ska = !va || excluded(g.nbr_src, ca, ea, sa, s);
        if (__syncthreads_and(ska)) continue;
        const int g0 = g.gidx[s], gl = g.glen[s];
        for (int base = 0; base < gl; base += kFarTile) {
            const int n = min(kFarTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sp[k] = g.pos64[g0 + base + k];
                sf[k] = src[g0 + base + k];
            }
            __syncthreads();
            if (!ska) {
#pragma unroll 4
                for (int k = 0; k < n; ++k) {
                    if (TRAC) pair_trac64(pa, na, sp[k], sf[k], xa, ya, za);
                    else pair_sl64(pa, sp[k], sf[k], xa, ya, za);
                }
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
    if (va) {
        double* o = partial + pr.poff + 3LL * mp * it.chunk + 3LL * (ta - pr.p0);
        o[0] = xa;
        o[1] = ya;
        o[2] = za;
    }
}

// ---------------------------------------------------------------- float-float (df64) far field
// Each value is an unevaluated sum hi + lo of two floats (about 48 significant bits). All
// arithmetic runs on the FP32 pipe (FMA for exact products), which GB300 issues 58x faster than
// FP64; per traction pair ~190 FP32 instructions. Used for the high-precision passes of the
// mixed-precision solve (right-hand side, refinement residuals, final single layer).
struct df {
    float h, l;
};

// __fmul_rn/__fadd_rn/__fsub_rn keep every rounding explicit: the compiler may not contract a
// product into a later addition, which would break the error-free transformations below.
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
    const df s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.h, -p);
    return quick_two_sum(p, fmaf(a.h, b.l, fmaf(a.l, b.h, e)));
}
// product left unnormalised (|lo| may reach a few ulp of hi): fine as an input to further
// products and to two_sum-based sums, and 3 instructions cheaper
__device__ __forceinline__ df df_mul_u(df a, df b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.h, -p);
    return {p, fmaf(a.h, b.l, fmaf(a.l, b.h, e))};
}
// a.a for a 3-vector of float-float components
__device__ __forceinline__ df df_sqr3(df a, df b, df c) {
    const float p0 = __fmul_rn(a.h, a.h), p1 = __fmul_rn(b.h, b.h), p2 = __fmul_rn(c.h, c.h);
    float lo = __fadd_rn(__fadd_rn(fmaf(a.h, a.h, -p0), fmaf(b.h, b.h, -p1)), fmaf(c.h, c.h, -p2));
    lo = fmaf(__fadd_rn(a.h, a.h), a.l, lo);
    lo = fmaf(__fadd_rn(b.h, b.h), b.l, lo);
    lo = fmaf(__fadd_rn(c.h, c.h), c.l, lo);
    const df s01 = two_sum(p0, p1);
    const df s = two_sum(s01.h, p2);
    return quick_two_sum(s.h, __fadd_rn(__fadd_rn(s.l, s01.l), lo));
}
// a*b + c*d + e*f with one renormalisation
__device__ __forceinline__ df df_dot3(df a, df b, df c, df d, df e, df f) {
    const float p0 = __fmul_rn(a.h, b.h), p1 = __fmul_rn(c.h, d.h), p2 = __fmul_rn(e.h, f.h);
    float lo = __fadd_rn(__fadd_rn(fmaf(a.h, b.h, -p0), fmaf(c.h, d.h, -p1)), fmaf(e.h, f.h, -p2));
    lo = fmaf(a.h, b.l, fmaf(a.l, b.h, lo));
    lo = fmaf(c.h, d.l, fmaf(c.l, d.h, lo));
    lo = fmaf(e.h, f.l, fmaf(e.l, f.h, lo));
    const df s01 = two_sum(p0, p1);
    const df s = two_sum(s01.h, p2);
    return quick_two_sum(s.h, __fadd_rn(__fadd_rn(s.l, s01.l), lo));
}
__device__ __forceinline__ df df_rsqrt(df x) {
    const float y = rsqrtf(x.h);
    const float yy = __fmul_rn(y, y);
    const float yye = fmaf(y, y, -yy);
    // x*y^2 = 1 - e, evaluated to double-float accuracy; one Newton step squares the error
    const float p = __fmul_rn(x.h, yy);
    const float pe = fmaf(x.h, yy, -p);
    const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), fmaf(x.h, yye, __fmul_rn(x.l, yy)));
    return quick_two_sum(y, __fmul_rn(__fmul_rn(0.5f, y), e));
}
__device__ __forceinline__ df df_sub(float4 a_h, float4 a_l, float4 b_h, float4 b_l, int k) {
    const float ah = k == 0 ? a_h.x : (k == 1 ? a_h.y : a_h.z);
    const float al = k == 0 ? a_l.x : (k == 1 ? a_l.y : a_l.z);
    const float bh = k == 0 ? b_h.x : (k == 1 ? b_h.y : b_h.z);
    const float bl = k == 0 ? b_l.x : (k == 1 ? b_l.y : b_l.z);
    const df s = two_sum(ah, -bh);
    return {s.h, __fadd_rn(s.l, __fsub_rn(al, bl))};  // nearly normalised; not renormalised
}
// accumulator: hi part by two_sum, lo parts summed and folded in at the end
__device__ __forceinline__ void df_acc(float& ah, float& al, df v) {
    const df s = two_sum(ah, v.h);
    ah = s.h;
    al = __fadd_rn(al, __fadd_rn(s.l, v.l));
}

template <bool TRAC>
__global__ void __launch_bounds__(kFarThreads) k_far_df(DevGeom g, const FarItem* __restrict__ items,
                                                       const float4* __restrict__ src, double* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ float4 sph[kFarTile], spl[kFarTile], sfh[kFarTile], sfl[kFarTile];
    const int ta = it.t0 + threadIdx.x;
    const bool va = ta < it.t1;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 ph = va ? g.pos32[ta] : z4, pl = va ? g.pos32lo[ta] : z4;
    float4 nh = z4, nl = z4;
    if (TRAC && va) {
        nh = g.nrm32[ta];
        nl = g.nrm32lo[ta];
    }
    const df n0{nh.x, nl.x}, n1{nh.y, nl.y}, n2{nh.z, nl.z};
    const int sa = va ? __float_as_int(ph.w) : -1;
    int ca = va ? g.nbr_start[sa] : 0, ea = va ? g.nbr_start[sa + 1] : 0;
    float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f, zh = 0.f, zl = 0.f;
    for (int s = it.s0; s < it.s1; ++s) {
        const bool ska = !va || excluded(g.nbr_src, ca, ea, sa, s);
        if (__syncthreads_and(ska)) continue;
        const int g0 = g.gidx[s], gl = g.glen[s];
        for (int base = 0; base < gl; base += kFarTile) {
            const int n = min(kFarTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sph[k] = g.pos32[g0 + base + k];
                spl[k] = g.pos32lo[g0 + base + k];
                sfh[k] = src[2 * (g0 + base + k)];
                sfl[k] = src[2 * (g0 + base + k) + 1];
            }
            __syncthreads();
            if (!ska) {
                for (int k = 0; k < n; ++k) {
                    const float4 qh = sph[k], ql = spl[k], fh = sfh[k], fl = sfl[k];
                    const df rx = df_sub(ph, pl, qh, ql, 0), ry = df_sub(ph, pl, qh, ql, 1),
                             rz = df_sub(ph, pl, qh, ql, 2);
                    const df f0{fh.x, fl.x}, f1{fh.y, fl.y}, f2{fh.z, fl.z};
                    const df r2 = df_sqr3(rx, ry, rz);
                    const df ri = df_rsqrt(r2);
                    const df rf = df_dot3(rx, f0, ry, f1, rz, f2);
                    if (TRAC) {
                        const df rn = df_dot3(rx, n0, ry, n1, rz, n2);
                        const df ri2 = df_mul_u(ri, ri);
                        const df k5 = df_mul(df_mul_u(rf, rn), df_mul_u(df_mul_u(ri2, ri2), ri));
                        df_acc(xh, xl, df_mul_u(k5, rx));
                        df_acc(yh, yl, df_mul_u(k5, ry));
                        df_acc(zh, zl, df_mul_u(k5, rz));
                    } else {
                        const df k3 = df_mul(rf, df_mul_u(df_mul_u(ri, ri), ri));
                        df_acc(xh, xl, df_add(df_mul_u(f0, ri), df_mul_u(k3, rx)));
                        df_acc(yh, yl, df_add(df_mul_u(f1, ri), df_mul_u(k3, ry)));
                        df_acc(zh, zl, df_add(df_mul_u(f2, ri), df_mul_u(k3, rz)));
                    }
                }
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
    if (va) {
        double* o = partial + pr.poff + 3LL * mp * it.chunk + 3LL * (ta - pr.p0);
        o[0] = double(xh) + double(xl);
        o[1] = double(yh) + double(yl);
        o[2] = double(zh) + double(zl);
    }
}

// sources as float-float pairs: src2[2i] = hi(x w c), src2[2i+1] = lo
__global__ void k_far_pack_df(DevGeom g, const double* __restrict__ x, double c, float4* __restrict__ s2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    if (g.active && !g.active[g.prob[g.sid[i]]]) return;
    const double w = g.weights[i] * c;
    const double f[3] = {x[3 * i] * w, x[3 * i + 1] * w, x[3 * i + 2] * w};
    float hi[3], lo[3];
    for (int k = 0; k < 3; ++k) {
        hi[k] = float(f[k]);
        lo[k] = float(f[k] - double(hi[k]));
    }
    s2[2 * i] = make_float4(hi[0], hi[1], hi[2], 0.f);
    s2[2 * i + 1] = make_float4(lo[0], lo[1], lo[2], 0.f);
}

__global__ void k_far_pack(DevGeom g, const double* __restrict__ x, double c, float4* __restrict__ s32,
                           double4* __restrict__ s64) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    if (g.active && !g.active[g.prob[g.sid[i]]]) return;
    const double w = g.weights[i] * c;
    const double fx = x[3 * i] * w, fy = x[3 * i + 1] * w, fz = x[3 * i + 2] * w;
    if (s32) s32[i] = make_float4(float(fx), float(fy), float(fz), 0.f);
    if (s64) s64[i] = make_double4(fx, fy, fz, 0.0);
}

template <typename Real>
__global__ void k_far_reduce(DevGeom g, const Real* __restrict__ partial, double pre, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    const int pb = g.prob[g.sid[i]];
    if (g.active && !g.active[pb]) return;
    const Problem pr = g.problems[pb];
    const long long mp = pr.p1 - pr.p0;
    const Real* base = partial + pr.poff + 3LL * (i - pr.p0);
    double sx = 0, sy = 0, sz = 0;
    for (int c = 0; c < pr.nchunks; ++c) {
        const Real* q = base + 3LL * mp * c;
        sx += double(q[0]);
        sy += double(q[1]);
        sz += double(q[2]);
    }
    out[3 * i] += pre * sx;
    out[3 * i + 1] += pre * sy;
    out[3 * i + 2] += pre * sz;
}

}  // namespace

int launch_far_pack(const DevGeom& g, const double* x, double c, float4* src32, double4* src64, bool fp32,
                    cudaStream_t st) {
    k_far_pack<<<(g.M + 255) / 256, 256, 0, st>>>(g, x, c, fp32 ? src32 : nullptr, fp32 ? nullptr : src64);
    return 1;
}

template <int TPT>
void launch_far32(const DevGeom& g, const FarItem* items, int nitems, bool trac, const float4* src32, float* partial,
                  cudaStream_t st) {
    if (trac) k_far32<true, TPT><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
    else k_far32<false, TPT><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
}

int launch_far_field(const DevGeom& g, const FarItem* items, int nitems, bool trac, bool fp32, const float4* src32,
                     const double4* src64, void* partial, cudaStream_t st, int tpt) {
    if (nitems <= 0) return 0;
    if (fp32) {
        float* pf = static_cast<float*>(partial);
        if (tpt == 1) launch_far32<1>(g, items, nitems, trac, src32, pf, st);
        else if (tpt == 4) launch_far32<4>(g, items, nitems, trac, src32, pf, st);
        else launch_far32<2>(g, items, nitems, trac, src32, pf, st);
    } else {
        if (trac) k_far64<true><<<nitems, kFarThreads, 0, st>>>(g, items, src64, static_cast<double*>(partial));
        else k_far64<false><<<nitems, kFarThreads, 0, st>>>(g, items, src64, static_cast<double*>(partial));
    }
    return 1;
}

int launch_far_pack_df(const DevGeom& g, const double* x, double c, float4* src2, cudaStream_t st) {
    k_far_pack_df<<<(g.M + 255) / 256, 256, 0, st>>>(g, x, c, src2);
    return 1;
}

int launch_far_field_df(const DevGeom& g, const FarItem* items, int nitems, bool trac, const float4* src2,
                        double* partial, cudaStream_t st) {
    if (nitems <= 0) return 0;
    if (trac) k_far_df<true><<<nitems, kFarThreads, 0, st>>>(g, items, src2, partial);
    else k_far_df<false><<<nitems, kFarThreads, 0, st>>>(g, items, src2, partial);
    return 1;
}

int launch_far_reduce(const DevGeom& g, const void* partial, bool fp32, double pre, double* out, cudaStream_t st) {
    const int blocks = (g.M + 255) / 256;
    if (fp32) k_far_reduce<float><<<blocks, 256, 0, st>>>(g, static_cast<const float*>(partial), pre, out);
    else k_far_reduce<double><<<blocks, 256, 0, st>>>(g, static_cast<const double*>(partial), pre, out);
    return 1;
}

}  // namespace smob
