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

template <bool TRAC>
__global__ void __launch_bounds__(kFarThreads) k_far32(DevGeom g, const FarItem* __restrict__ items,
                                                      const float4* __restrict__ src, float* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ float4 sp[kFarTile];
    __shared__ float4 sf[kFarTile];
    const int ta = it.t0 + threadIdx.x, tb = ta + kFarThreads;
    const bool va = ta < it.t1, vb = tb < it.t1;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pa = va ? g.pos32[ta] : z4, pb = vb ? g.pos32[tb] : z4;
    float4 na = z4, nb = z4;
    if (TRAC) {
        if (va) na = g.nrm32[ta];
        if (vb) nb = g.nrm32[tb];
    }
    const int sa = va ? __float_as_int(pa.w) : -1, sb = vb ? __float_as_int(pb.w) : -1;
    int ca = va ? g.nbr_start[sa] : 0, ea = va ? g.nbr_start[sa + 1] : 0;
    int cb = vb ? g.nbr_start[sb] : 0, eb = vb ? g.nbr_start[sb + 1] : 0;
    float xa = 0.f, ya = 0.f, za = 0.f, xb = 0.f, yb = 0.f, zb = 0.f;
    for (int s = it.s0; s < it.s1; ++s) {
        const bool ska = !va || excluded(g.nbr_src, ca, ea, sa, s);
        const bool skb = !vb || excluded(g.nbr_src, cb, eb, sb, s);
        if (__syncthreads_and(ska && skb)) continue;
        const int g0 = g.gidx[s], gl = g.glen[s];
        for (int base = 0; base < gl; base += kFarTile) {
            const int n = min(kFarTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sp[k] = g.pos32[g0 + base + k];
                sf[k] = src[g0 + base + k];
            }
            __syncthreads();
            if (!ska && !skb) {
#pragma unroll 4
                for (int k = 0; k < n; ++k) {
                    const float4 q = sp[k], f = sf[k];
                    if (TRAC) {
                        pair_trac32(pa, na, q, f, xa, ya, za);
                        pair_trac32(pb, nb, q, f, xb, yb, zb);
                    } else {
                        pair_sl32(pa, q, f, xa, ya, za);
                        pair_sl32(pb, q, f, xb, yb, zb);
                    }
                }
            } else if (!ska) {
                for (int k = 0; k < n; ++k) {
                    if (TRAC) pair_trac32(pa, na, sp[k], sf[k], xa, ya, za);
                    else pair_sl32(pa, sp[k], sf[k], xa, ya, za);
                }
            } else if (!skb) {
                for (int k = 0; k < n; ++k) {
                    if (TRAC) pair_trac32(pb, nb, sp[k], sf[k], xb, yb, zb);
                    else pair_sl32(pb, sp[k], sf[k], xb, yb, zb);
                }
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
    float* out = partial + pr.poff + 3LL * mp * it.chunk;
    if (va) {
        float* o = out + 3LL * (ta - pr.p0);
        o[0] = xa;
        o[1] = ya;
        o[2] = za;
    }
    if (vb) {
        float* o = out + 3LL * (tb - pr.p0);
        o[0] = xb;
        o[1] = yb;
        o[2] = zb;
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

int launch_far_field(const DevGeom& g, const FarItem* items, int nitems, bool trac, bool fp32, const float4* src32,
                     const double4* src64, void* partial, cudaStream_t st) {
    if (nitems <= 0) return 0;
    if (fp32) {
        if (trac) k_far32<true><<<nitems, kFarThreads, 0, st>>>(g, items, src32, static_cast<float*>(partial));
        else k_far32<false><<<nitems, kFarThreads, 0, st>>>(g, items, src32, static_cast<float*>(partial));
    } else {
        if (trac) k_far64<true><<<nitems, kFarThreads, 0, st>>>(g, items, src64, static_cast<double*>(partial));
        else k_far64<false><<<nitems, kFarThreads, 0, st>>>(g, items, src64, static_cast<double*>(partial));
    }
    return 1;
}

int launch_far_reduce(const DevGeom& g, const void* partial, bool fp32, double pre, double* out, cudaStream_t st) {
    const int blocks = (g.M + 255) / 256;
    if (fp32) k_far_reduce<float><<<blocks, 256, 0, st>>>(g, static_cast<const float*>(partial), pre, out);
    else k_far_reduce<double><<<blocks, 256, 0, st>>>(g, static_cast<const double*>(partial), pre, out);
    return 1;
}

}  // namespace smob
