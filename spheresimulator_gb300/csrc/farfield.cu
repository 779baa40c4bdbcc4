// farfield.cu — all-pairs Stokes single-layer / traction far field.
//
// Replaces the STKFMM far-field evaluations of BIE/SphereSTKSHOperator.cpp:273-303 (PVel)
// and :354-446 (Traction, dotted with the target normal) by summation over all pairs:
//   SL:        u(x) = 1/(8 pi) sum_y [ f/r + (r.f) r / r^3 ]
//   traction:  t(x) = -3/(4 pi) sum_y r (r.f)(r.n_x) / r^5,      r = x - y, f = w_y * density_y * c
// Sources on the target's own sphere are skipped (the reference adds then subtracts them,
// :306-351 and :375-433) and so are sources on the target's near-pair spheres (the
// reference subtracts their direct sum and adds the spectral value, :575-695); both are
// accounted for spectrally by the sphere and near kernels, so the sum here is exactly the
// remaining smooth-quadrature part.
//
// Work decomposition: one CTA per work item = (block of targets of one problem) x (chunk of
// source spheres of the same problem). Sources are staged per sphere in shared memory; each thread
// owns 1, 2 or 4 targets in FP32 (scalar, or packed FP32x2 lanes; the autotuner picks), 2 in
// float-float (packed) and 1 in FP64. The several-right-hand-side kernels run one problem's work
// items for up to 8 (FP32) or 4 (float-float) copies of it at once, evaluating each pair's geometry
// once. A per-thread merge cursor over the sorted near-pair list decides per source sphere whether
// the thread's target skips it. The FP32 and float-float kernels also vote per source sphere for its
// coarse equivalent sources when every target of the CTA is far enough (see the coarse section
// below); the CTA stages the grid sources, one coarse level, or nothing when every target skips.
// Partial sums go to [problem][chunk][point][3] and a second kernel reduces the chunks in
// fixed order, so results do not depend on scheduling or on other problems in the batch.
#include "smob_internal.h"
#include "df.h"
#include "tc_sm100.h"

namespace smob {

namespace {

// One MUFU instruction each (PTX rsqrt/rcp .approx.ftz): plain rsqrtf adds a fix-up for denormal
// arguments, which a squared pair distance never is. 1/r^2 from its own MUFU spares the FMA pipes
// the ri*ri product that the pair would otherwise spend on it.
__device__ __forceinline__ float rsqrt_mufu(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_mufu(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// r^-5 of a squared distance as 2^(-2.5 log2 r^2): two MUFU instructions and one multiply, where
// rsqrt, rcp and q*q*ri take two MUFU and two multiplies (the traction pair needs no plain 1/r).
// Relative error ~5e-7 (lg2.approx's absolute error times 2.5 ln 2, plus ex2.approx's 2 ulp).
__device__ __forceinline__ float rpow5_mufu(float r2) {
    float l, y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(r2));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-2.5f * l));
    return y;
}

__device__ __forceinline__ void pair_trac32(const float4& t, const float4& n, const float4& s, const float4& f,
                                            float& ax, float& ay, float& az) {
    const float rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float ri5 = rpow5_mufu(r2);
    const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
    const float rn = fmaf(rx, n.x, fmaf(ry, n.y, rz * n.z));
    const float k = (rf * rn) * ri5;
    ax = fmaf(k, rx, ax);
    ay = fmaf(k, ry, ay);
    az = fmaf(k, rz, az);
}

__device__ __forceinline__ void pair_sl32(const float4& t, const float4& s, const float4& f, float& ax, float& ay,
                                          float& az) {
    const float rx = t.x - s.x, ry = t.y - s.y, rz = t.z - s.z;
    const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
    const float ri = rsqrt_mufu(r2), q = rcp_mufu(r2);
    const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
    const float k = rf * (q * ri);
    ax = fmaf(f.x, ri, fmaf(k, rx, ax));
    ay = fmaf(f.y, ri, fmaf(k, ry, ay));
    az = fmaf(f.z, ri, fmaf(k, rz, az));
}

__device__ __forceinline__ void pair_trac64(const double4_32a& t, const double4_32a& n, const double4_32a& s, const double4_32a& f,
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

__device__ __forceinline__ void pair_sl64(const double4_32a& t, const double4_32a& s, const double4_32a& f, double& ax,
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

// ---------------------------------------------------------------- coarse equivalent sources (FP32)
// For a well-separated pair of spheres the far field of the source sphere's grid sources equals that
// of equivalent sources on a coarser grid of the same sphere (order pe: the sources projected onto
// the harmonics of degree <= pe and re-weighted with the coarse quadrature) to ~(a_s / r_min)^(pe+1)
// relative, r_min the distance from the source centre to the nearest target point. Each target votes
// per source sphere for the coarsest level within the tolerance; the CTA takes the finest vote, or
// the fine sources (with the exclusions) when a target skips the sphere.
constexpr unsigned kBitFine = 1u << kCoarseLevels;  // the sphere's own grid sources
constexpr unsigned kBitSkip = 2u << kCoarseLevels;  // own sphere or near pair of some target

__device__ __forceinline__ unsigned level_bit(const DevGeom& g, const CoarseSet& cs, int t, int s) {
    if (cs.ncent == 0) return kBitFine;
    const int4* L = cs.clev + s * kCoarseLevels;
    if (__ldg(&L[0].x) == 0) return kBitFine;
    const float4 ct = __ldg(g.sph32 + t), cs4 = __ldg(g.sph32 + s);
    const float dx = ct.x - cs4.x, dy = ct.y - cs4.y, dz = ct.z - cs4.z;
    const float rmin = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - ct.w;
    const float as = cs4.w;
    if (!(rmin > as)) return kBitFine;
    const float need = cs.clog_eps / __logf(as / rmin) + cs.cmargin;
#pragma unroll 1
    for (int l = 0; l < kCoarseLevels; ++l) {
        const int pe = __ldg(&L[l].x);
        if (pe == 0) break;
        if (float(pe) >= need) return 1u << l;
    }
    return kBitFine;
}

// Coarse-target level of the far pair (target sphere t, source sphere s): the index of the coarsest
// built level of t with pe >= clog_eps / log(a_t / (|c_t - c_s| - a_s)) + ctmargin, if that level has
// at most kCoarseTargetNum / kCoarseTargetDen of t's grid points; else -1 (grid targets). The grid
// kernels skip exactly the pairs for which this is >= 0 and the coarse-target kernel evaluates exactly
// those (both call this function on the same arguments). Near pairs and t == s are excluded by the
// callers.
__device__ __forceinline__ int tgt_level(const DevGeom& g, const CoarseSet& cs, int t, int s) {
    if (!cs.ctgt || cs.ncent == 0) return -1;
    const int4* L = cs.clev + t * kCoarseLevels;
    if (__ldg(&L[0].x) == 0) return -1;
    const float4 ct = __ldg(g.sph32 + t), cs4 = __ldg(g.sph32 + s);
    const float dx = ct.x - cs4.x, dy = ct.y - cs4.y, dz = ct.z - cs4.z;
    const float rmin = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - cs4.w;
    const float at = ct.w;
    if (!(rmin > at)) return -1;
    const float need = cs.clog_eps / __logf(at / rmin) + cs.ctmargin;
    const int cap = __ldg(g.glen + t) * kCoarseTargetNum;
#pragma unroll 1
    for (int l = 0; l < kCoarseLevels; ++l) {
        const int4 Ll = __ldg(&L[l]);
        if (Ll.x == 0) break;
        if (float(Ll.x) >= need) return Ll.z * kCoarseTargetDen <= cap ? l : -1;
    }
    return -1;
}

// CTA-wide OR of one vote per thread (per-warp slots, double-buffered by parity: one barrier); NT threads
template <int NT = kFarThreads>
__device__ __forceinline__ unsigned cta_or(unsigned v, unsigned (*slots)[NT / 32], int parity) {
    v = __reduce_or_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) slots[parity][threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned r = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) r |= slots[parity][w];
    return r;
}

// the CTA's source range for sphere s from its votes: fine grid points or one coarse level (FP32 set);
// targets that skip the sphere do not vote, and the others may take coarse sources (a masked loop)
__device__ __forceinline__ bool pick_sources(const DevGeom& g, int s, unsigned votes, const float4* src,
                                             const float4*& P, const float4*& F, int& g0, int& gl) {
    const unsigned lv = votes & ~kBitSkip;
    const bool coarse = !(lv & kBitFine);
    if (coarse) {
        const int4 L = g.cs32.clev[s * kCoarseLevels + (31 - __clz(lv))];
        P = g.cs32.cpos32;
        F = g.cs32.csrc;
        g0 = L.y;
        gl = L.z;
    } else {
        P = g.pos32;
        F = src;
        g0 = g.gidx[s];
        gl = g.glen[s];
    }
    return coarse;
}

// f_e = coarse map x weighted sources: per (p, pe) map a GEMM [N_e x N_g] x [N_g x 3 per sphere]. A CTA
// computes kCoarseTileNodes coarse nodes of up to 8 spheres; its 4 groups of 128 threads take interleaved
// slices of 16 fine nodes (map rows and the spheres' sources staged in shared memory), thread (sphere
// t / 16, nodes t % 16 + 16 i) of a group keeps kCgNi x 3 accumulators, and the groups' sums are added
// in a fixed order at the end.
constexpr int kCgNodes = kCoarseTileNodes, kCgSph = 8, kCgK = 16, kCgGroups = 4;
constexpr int kCgNi = kCgNodes / 16;  // coarse nodes per thread
__global__ void __launch_bounds__(128 * kCgGroups) k_coarse_src(DevGeom g, const float4* __restrict__ src) {
    const CoarseSet& cs = g.cs32;
    const int4 d = cs.cdesc[blockIdx.x];
    const int4 G = cs.cgrp[d.x];
    const int k0 = d.y, ne = d.w, ng = G.y, cnt = G.z;
    __shared__ float Ms[kCgGroups][kCgK][kCgNodes];
    __shared__ float4 Fs[kCgGroups][kCgK][kCgSph];
    __shared__ float red[kCgGroups - 1][3 * kCgNi][128];
    __shared__ int sbase[kCgSph], sout[kCgSph];
    __shared__ unsigned char sact[kCgSph];
    const int grp = threadIdx.x >> 7, t = threadIdx.x & 127;
    if (threadIdx.x < kCgSph) {
        int sb = 0, so = 0;
        unsigned char a = 0;
        if (threadIdx.x < ne) {
            const int2 e = cs.gent[d.z + threadIdx.x];
            sb = g.gidx[e.x];
            so = e.y;
            a = (g.active && !g.active[g.prob[e.x]]) ? 0 : 1;
        }
        sbase[threadIdx.x] = sb;
        sout[threadIdx.x] = so;
        sact[threadIdx.x] = a;
    }
    __syncthreads();
    const int si = t >> 4, ni = t & 15;
    float acc[kCgNi][3];
#pragma unroll
    for (int i = 0; i < kCgNi; ++i) acc[i][0] = acc[i][1] = acc[i][2] = 0.f;
    const float* __restrict__ map = cs.cmap + G.x;
    for (int jb = 0; jb < ng; jb += kCgK * kCgGroups) {
        const int j0 = jb + grp * kCgK;  // this group's slice
#pragma unroll
        for (int r = 0; r < kCgK * kCgNodes / 128; ++r) {
            const int idx = t + 128 * r, jj = idx / kCgNodes, kk = idx % kCgNodes;
            Ms[grp][jj][kk] =
                (j0 + jj < ng && k0 + kk < cnt) ? __ldg(map + (long long)(j0 + jj) * cnt + k0 + kk) : 0.f;
        }
        if (t < kCgK * kCgSph) {
            const int jj = t / kCgSph, ss = t % kCgSph;
            Fs[grp][jj][ss] = (j0 + jj < ng && ss < ne) ? src[sbase[ss] + j0 + jj] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < kCgK; ++jj) {
            const float4 f = Fs[grp][jj][si];
#pragma unroll
            for (int i = 0; i < kCgNi; ++i) {
                const float m = Ms[grp][jj][ni + 16 * i];
                acc[i][0] = fmaf(m, f.x, acc[i][0]);
                acc[i][1] = fmaf(m, f.y, acc[i][1]);
                acc[i][2] = fmaf(m, f.z, acc[i][2]);
            }
        }
        __syncthreads();
    }
    if (grp > 0) {
#pragma unroll
        for (int i = 0; i < kCgNi; ++i)
#pragma unroll
            for (int c = 0; c < 3; ++c) red[grp - 1][3 * i + c][t] = acc[i][c];
    }
    __syncthreads();
    if (grp == 0 && si < ne && sact[si]) {
#pragma unroll
        for (int i = 0; i < kCgNi; ++i) {
#pragma unroll
            for (int q = 0; q < kCgGroups - 1; ++q)
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[i][c] += red[q][3 * i + c][t];
            const int k = k0 + ni + 16 * i;
            if (k < cnt) cs.csrc[sout[si] + k] = make_float4(acc[i][0], acc[i][1], acc[i][2], 0.f);
        }
    }
}

// The FP32 set's strengths on the tcgen05 tensor cores: per (p, pe) map the GEMM
//   D [128 coarse nodes x 48] = A [128 x N_g] . B [48 x N_g]^T,
// A = the transposed map's rows (coarse node k: its N_g fine-node weights), B = the sources of 16
// spheres, one row per (sphere, component). K runs over the fine nodes in chunks of 32 TF32 values,
// both operands as TF32 high and low parts (3xTF32: hi.hi + hi.lo + lo.hi, about FP32 accuracy): A is
// copied from its pre-split tiles (cs.cmapA, coalesced float4 loads), B gathered and split by the
// threads. One thread issues the chunk's 12 MMAs, commits them to an mbarrier and waits (bounded);
// D stays in tensor memory over the chunks (48 of 64 allocated columns). The K chunks are split over
// kCsTcSplit CTAs (grid y) so a tile's chunks run side by side: each CTA loads its D rows and writes
// them as partial sums (cs.cpart[split]); the last CTA of the tile to finish (a counter per tile,
// after a memory fence) adds the splits in fixed order and writes the 16 spheres' strengths. Every
// D element is the same sum whichever spheres share its tile and whichever CTA finishes last, so a
// problem's strengths do not depend on the batch or the schedule.
constexpr int kCsTcSph = kCoarseTcSph, kCsTcN = 3 * kCsTcSph, kCsTcK = 32;
static_assert(kCoarseTcNodes == 128, "one M = 128 MMA tile per CTA");
constexpr int kCsTcABytes = 128 * kCsTcK * 4, kCsTcBBytes = kCsTcN * kCsTcK * 4;
constexpr int kCsTcSmem = 2 * kCsTcABytes + 2 * kCsTcBBytes;  // A hi, A lo, B hi, B lo: 44 KB
constexpr long long kCsTcWaitPolls = 1LL << 22;
static_assert(kCoarseTcSplit >= 1, "at least one split");
__global__ void __launch_bounds__(128) k_coarse_src_tc(DevGeom g, const float4* __restrict__ src) {
    const CoarseSet& cs = g.cs32;
    const int4 d = cs.cdesc_tc[blockIdx.x];
    const int split = blockIdx.y;
    const int4 G = cs.cgrp[d.x];
    const int k0 = d.y, ne = d.w, ng = G.y, cnt = G.z;
    extern __shared__ __align__(1024) unsigned char cs_smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ int s_fail;
    __shared__ int sbase[kCsTcSph], sout[kCsTcSph];
    __shared__ unsigned char sact[kCsTcSph];
    __shared__ int s_last;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid < kCsTcSph) {
        int sb = 0, so = 0;
        unsigned char a = 0;
        if (tid < ne) {
            const int2 e = cs.gent[d.z + tid];
            sb = g.gidx[e.x];
            so = e.y;
            a = (g.active && !g.active[g.prob[e.x]]) ? 0 : 1;
        }
        sbase[tid] = sb;
        sout[tid] = so;
        sact[tid] = a;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_fence_init();
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    constexpr uint32_t idesc = tc::idesc_tf32(128, kCsTcN);
    unsigned char* sAh = cs_smem;
    unsigned char* sAl = cs_smem + kCsTcABytes;
    unsigned char* sBh = cs_smem + 2 * kCsTcABytes;
    unsigned char* sBl = sBh + kCsTcBBytes;
    const int krow = k0 + tid;  // this thread's D row (coarse node)
    const bool rvalid = krow < cnt;
    const int nck = (ng + kCsTcK - 1) / kCsTcK;
    const int ch0 = split * nck / kCoarseTcSplit, ch1 = (split + 1) * nck / kCoarseTcSplit;  // this CTA's chunks
    // this tile's A chunks: [chunk][hi, lo][128 x 32 in core-matrix order]
    const float4* __restrict__ At = cs.cmapA + (G.w + (long long)(k0 / 128) * nck * 2 * 128 * kCsTcK) / 4;
    unsigned phase = 0;
    bool failed = false;
    for (int ch = ch0; ch < ch1; ++ch) {
        const int j0 = ch * kCsTcK;
        // A: the chunk's pre-split tiles, hi then lo, straight copies
        {
            const float4* src_h = At + (long long)ch * 2 * (kCsTcABytes / 16);
            const float4* src_l = src_h + kCsTcABytes / 16;
#pragma unroll
            for (int v = tid; v < kCsTcABytes / 16; v += 128) {
                reinterpret_cast<float4*>(sAh)[v] = __ldg(src_h + v);
                reinterpret_cast<float4*>(sAl)[v] = __ldg(src_l + v);
            }
        }
        // B: rows 3 s + c (sphere s of the tile, component c), 32 fine nodes
        for (int v = tid; v < kCsTcSph * kCsTcK; v += 128) {
            const int si = v / kCsTcK, jj = v % kCsTcK, j = j0 + jj;
            const float4 f = (si < ne && j < ng) ? src[sbase[si] + j] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float fc[3] = {f.x, f.y, f.z};
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                // the low part rounded to TF32 as well (the MMA would truncate it), like the A tiles
                const float h = tc::tf32_hi(fc[cc]), l = tc::tf32_hi(fc[cc] - h);
                const uint32_t off = tc::kmajor_offset(3 * si + cc, jj, kCsTcK);
                *reinterpret_cast<float*>(sBh + off) = h;
                *reinterpret_cast<float*>(sBl + off) = l;
            }
        }
        tc::fence_smem_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t ah0 = tc::smem_u32(sAh), al0 = tc::smem_u32(sAl);
            const uint32_t bh0 = tc::smem_u32(sBh), bl0 = tc::smem_u32(sBl);
            constexpr uint32_t sbo = (kCsTcK / 4) * 128;
#pragma unroll
            for (int ks = 0; ks < kCsTcK / 8; ++ks) {
                const uint32_t o = ks * 256;
                const uint64_t ah = tc::sdesc(ah0 + o, 128, sbo), al = tc::sdesc(al0 + o, 128, sbo);
                const uint64_t bh = tc::sdesc(bh0 + o, 128, sbo), bl = tc::sdesc(bl0 + o, 128, sbo);
                tc::mma_tf32(tmem, ah, bh, idesc, ch > ch0 || ks > 0);
                tc::mma_tf32(tmem, ah, bl, idesc, true);
                tc::mma_tf32(tmem, al, bh, idesc, true);
            }
            tc::mma_commit(&mbar);
            if (!tc::mbar_wait_bounded(&mbar, phase, kCsTcWaitPolls)) s_fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        if (s_fail) {
            failed = true;
            break;
        }
    }
    // this split's partial sums (zeros for a split without chunks), then the tile's last CTA
    float4* __restrict__ part = cs.cpart + (long long)split * cs.ncoarse32;
    if (!failed) {
        float da[32], db[32];
        if (ch1 > ch0) {
            tc::fence_after_sync();
            const uint32_t lane_base = uint32_t(warp * 32) << 16;
            tc::tmem_ld_32x32b_x32(tmem + lane_base, da);       // columns 0-31
            tc::tmem_ld_32x32b_x32(tmem + 32 + lane_base, db);  // columns 32-63 (48-63 unused)
        } else {
#pragma unroll
            for (int q = 0; q < 32; ++q) da[q] = db[q] = 0.f;
        }
        if (rvalid) {
#pragma unroll
            for (int si = 0; si < kCsTcSph; ++si) {
                if (si >= ne || !sact[si]) continue;
                float o[3];
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) {
                    const int col = 3 * si + cc;
                    o[cc] = col < 32 ? da[col] : db[col - 32];
                }
                part[sout[si] + krow] = make_float4(o[0], o[1], o[2], 0.f);
            }
        }
    } else if (tid == 0 && g.err) {
        atomicExch(g.err, 1);
    }
    // every CTA of the tile counts itself once (also a failed one, whose results are void anyway)
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        unsigned* cnt_p = cs.ctile_count + blockIdx.x;
        s_last = atomicAdd(cnt_p, 1u) == unsigned(kCoarseTcSplit - 1) ? 1 : 0;
        if (s_last) *cnt_p = 0u;  // ready for the next pass
    }
    __syncthreads();
    if (s_last && rvalid) {
        __threadfence();
#pragma unroll 1
        for (int si = 0; si < ne; ++si) {
            if (!sact[si]) continue;
            const long long q = sout[si] + krow;
            float4 t = __ldcg(cs.cpart + q);
#pragma unroll
            for (int sp = 1; sp < kCoarseTcSplit; ++sp) {
                const float4 v = __ldcg(cs.cpart + (long long)sp * cs.ncoarse32 + q);
                t.x += v.x;
                t.y += v.y;
                t.z += v.z;
            }
            cs.csrc[q] = make_float4(t.x, t.y, t.z, 0.f);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 64);
    }
}

// The float-float set's strengths: the same GEMM tiles in float-float arithmetic on the FP32 pipes
// (the FP64 pipe issues 1/58 of their rate): maps stored as (hi, lo) float pairs, sources as the hi/lo
// float4 pairs of the grid, products by df_mul_u and sums by df_acc (~2^-44 relative to the sum of
// |terms|), two split-K groups of 128 threads added as float-float pairs; each strength is stored as a
// normalised hi/lo float pair like the grid sources.
constexpr int kCgGroupsD = 2;
__global__ void __launch_bounds__(128 * kCgGroupsD) k_coarse_src_df(DevGeom g, const float4* __restrict__ src2) {
    const CoarseSet& cs = g.cshp;
    const int4 d = cs.cdesc[blockIdx.x];
    const int4 G = cs.cgrp[d.x];
    const int k0 = d.y, ne = d.w, ng = G.y, cnt = G.z;
    __shared__ float2 Ms[kCgGroupsD][kCgK][kCgNodes];
    __shared__ float4 Fh[kCgGroupsD][kCgK][kCgSph], Fl[kCgGroupsD][kCgK][kCgSph];
    __shared__ float2 red[kCgGroupsD - 1][3 * kCgNi][128];
    __shared__ int sbase[kCgSph], sout[kCgSph];
    __shared__ unsigned char sact[kCgSph];
    const int grp = threadIdx.x >> 7, t = threadIdx.x & 127;
    if (threadIdx.x < kCgSph) {
        int sb = 0, so = 0;
        unsigned char a = 0;
        if (threadIdx.x < ne) {
            const int2 e = cs.gent[d.z + threadIdx.x];
            sb = g.gidx[e.x];
            so = e.y;
            a = (g.active && !g.active[g.prob[e.x]]) ? 0 : 1;
        }
        sbase[threadIdx.x] = sb;
        sout[threadIdx.x] = so;
        sact[threadIdx.x] = a;
    }
    __syncthreads();
    const int si = t >> 4, ni = t & 15;
    float ah[kCgNi][3], al[kCgNi][3];
#pragma unroll
    for (int i = 0; i < kCgNi; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) ah[i][c] = al[i][c] = 0.f;
    const float2* __restrict__ map = cs.cmapf2 + G.x;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int jb = 0; jb < ng; jb += kCgK * kCgGroupsD) {
        const int j0 = jb + grp * kCgK;
#pragma unroll
        for (int r = 0; r < kCgK * kCgNodes / 128; ++r) {
            const int idx = t + 128 * r, jj = idx / kCgNodes, kk = idx % kCgNodes;
            Ms[grp][jj][kk] = (j0 + jj < ng && k0 + kk < cnt) ? __ldg(map + (long long)(j0 + jj) * cnt + k0 + kk)
                                                              : make_float2(0.f, 0.f);
        }
        if (t < kCgK * kCgSph) {
            const int jj = t / kCgSph, ss = t % kCgSph;
            const bool in = j0 + jj < ng && ss < ne;
            Fh[grp][jj][ss] = in ? src2[2LL * (sbase[ss] + j0 + jj)] : z4;
            Fl[grp][jj][ss] = in ? src2[2LL * (sbase[ss] + j0 + jj) + 1] : z4;
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < kCgK; ++jj) {
            const float4 fh = Fh[grp][jj][si], fl = Fl[grp][jj][si];
#pragma unroll
            for (int i = 0; i < kCgNi; ++i) {
                const float2 m = Ms[grp][jj][ni + 16 * i];
                const df1 mm{m.x, m.y};
                df_acc(ah[i][0], al[i][0], df_mul_u(mm, df1{fh.x, fl.x}));
                df_acc(ah[i][1], al[i][1], df_mul_u(mm, df1{fh.y, fl.y}));
                df_acc(ah[i][2], al[i][2], df_mul_u(mm, df1{fh.z, fl.z}));
            }
        }
        __syncthreads();
    }
    if (grp > 0) {
#pragma unroll
        for (int i = 0; i < kCgNi; ++i)
#pragma unroll
            for (int c = 0; c < 3; ++c) red[grp - 1][3 * i + c][t] = make_float2(ah[i][c], al[i][c]);
    }
    __syncthreads();
    if (grp == 0 && si < ne && sact[si]) {
#pragma unroll
        for (int i = 0; i < kCgNi; ++i) {
            float o[3], ol[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
#pragma unroll
                for (int q = 0; q < kCgGroupsD - 1; ++q) {
                    const float2 v = red[q][3 * i + c][t];
                    df_acc(ah[i][c], al[i][c], df1{v.x, v.y});
                }
                const df1 s = two_sum(ah[i][c], al[i][c]);  // normalised: lo within half an ulp of hi
                o[c] = s.h;
                ol[c] = s.l;
            }
            const int k = k0 + ni + 16 * i;
            if (k < cnt) {
                cs.csrc[2LL * (sout[si] + k)] = make_float4(o[0], o[1], o[2], 0.f);
                cs.csrc[2LL * (sout[si] + k) + 1] = make_float4(ol[0], ol[1], ol[2], 0.f);
            }
        }
    }
}

// ---------------------------------------------------------------- packed FP32x2 far field
// Blackwell issues two FP32 lanes per FFMA2/FADD2/FMUL2 instruction (__ffma2_rn & co., same
// per-component rounding as the scalar forms). Targets are packed two per float2; each staged
// source is stored pre-duplicated, (x,x,y,y) (z,z,fx,fx) (fy,fy,fz,fz), so three 128-bit shared
// loads give the six broadcast operands. Per pair: ~10 packed instructions + two MUFU instructions.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

template <bool TRAC>
__device__ __forceinline__ void pair_x2(const float2& tx, const float2& ty, const float2& tz, const float2& nx,
                                        const float2& ny, const float2& nz, const float4& A, const float4& B,
                                        const float4& C, float2& ax, float2& ay, float2& az) {
    const float2 rx = __fadd2_rn(tx, f2(-A.x, -A.y));
    const float2 ry = __fadd2_rn(ty, f2(-A.z, -A.w));
    const float2 rz = __fadd2_rn(tz, f2(-B.x, -B.y));
    const float2 r2 = __ffma2_rn(rx, rx, __ffma2_rn(ry, ry, __fmul2_rn(rz, rz)));
    const float2 rf = __ffma2_rn(rx, f2(B.z, B.w), __ffma2_rn(ry, f2(C.x, C.y), __fmul2_rn(rz, f2(C.z, C.w))));
    if (TRAC) {
        const float2 ri5 = f2(rpow5_mufu(r2.x), rpow5_mufu(r2.y));
        const float2 rn = __ffma2_rn(rx, nx, __ffma2_rn(ry, ny, __fmul2_rn(rz, nz)));
        const float2 k = __fmul2_rn(__fmul2_rn(rf, rn), ri5);
        ax = __ffma2_rn(k, rx, ax);
        ay = __ffma2_rn(k, ry, ay);
        az = __ffma2_rn(k, rz, az);
    } else {
        const float2 ri = f2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y)), q = f2(rcp_mufu(r2.x), rcp_mufu(r2.y));
        const float2 k = __fmul2_rn(rf, __fmul2_rn(q, ri));
        ax = __ffma2_rn(f2(B.z, B.w), ri, __ffma2_rn(k, rx, ax));
        ay = __ffma2_rn(f2(C.x, C.y), ri, __ffma2_rn(k, ry, ay));
        az = __ffma2_rn(f2(C.z, C.w), ri, __ffma2_rn(k, rz, az));
    }
}

// NPK float2 packs = 2*NPK targets per thread; a work item covers kFarThreads * 2 * NPK targets
template <bool TRAC, int NPK>
__global__ void __launch_bounds__(kFarThreads) k_far32x2(DevGeom g, const FarItem* __restrict__ items,
                                                        const float4* __restrict__ src, float* __restrict__ partial) {
    constexpr int T = 2 * NPK;
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ float4 sA[kFarTile32], sB[kFarTile32], sC[kFarTile32];
    __shared__ unsigned votes_buf[2][kFarThreads / 32];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 TX[NPK], TY[NPK], TZ[NPK], NX[NPK], NY[NPK], NZ[NPK], AX[NPK], AY[NPK], AZ[NPK];
    int sid[T], cur[T], end[T];
    bool val[T];
#pragma unroll
    for (int q = 0; q < NPK; ++q) {
        float4 P[2], Nn[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = 2 * q + h;
            const int t = it.t0 + threadIdx.x + u * kFarThreads;
            val[u] = t < it.t1;
            P[h] = val[u] ? g.pos32[t] : z4;
            Nn[h] = (TRAC && val[u]) ? g.nrm32[t] : z4;
            sid[u] = val[u] ? __float_as_int(P[h].w) : -1;
            cur[u] = val[u] ? g.nbr_start[sid[u]] : 0;
            end[u] = val[u] ? g.nbr_start[sid[u] + 1] : 0;
        }
        TX[q] = f2(P[0].x, P[1].x);
        TY[q] = f2(P[0].y, P[1].y);
        TZ[q] = f2(P[0].z, P[1].z);
        NX[q] = f2(Nn[0].x, Nn[1].x);
        NY[q] = f2(Nn[0].y, Nn[1].y);
        NZ[q] = f2(Nn[0].z, Nn[1].z);
        AX[q] = AY[q] = AZ[q] = f2(0.f, 0.f);
    }
    int parity = 0;
    for (int s = it.s0; s < it.s1; ++s, parity ^= 1) {
        bool sk[T];
        bool none = true;
        unsigned vote = 0;
#pragma unroll
        for (int u = 0; u < T; ++u) {
            sk[u] = !val[u] || excluded(g.nbr_src, cur[u], end[u], sid[u], s) || tgt_level(g, g.cs32, sid[u], s) >= 0;
            none = none && !sk[u];
            if (val[u]) vote |= sk[u] ? kBitSkip : level_bit(g, g.cs32, sid[u], s);
        }
        const unsigned votes = cta_or(vote, votes_buf, parity);
        if (!(votes & ~kBitSkip)) continue;  // every target skips this sphere
        const float4 *SP, *SF;
        int g0, gl;
        pick_sources(g, s, votes, src, SP, SF, g0, gl);
        for (int base = 0; base < gl; base += kFarTile32) {
            const int n = min(kFarTile32, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                const float4 p = SP[g0 + base + k], f = SF[g0 + base + k];
                sA[k] = make_float4(p.x, p.x, p.y, p.y);
                sB[k] = make_float4(p.z, p.z, f.x, f.x);
                sC[k] = make_float4(f.y, f.y, f.z, f.z);
            }
            __syncthreads();
            if (none) {
#pragma unroll 4
                for (int k = 0; k < n; ++k) {
                    const float4 A = sA[k], B = sB[k], C = sC[k];
#pragma unroll
                    for (int q = 0; q < NPK; ++q)
                        pair_x2<TRAC>(TX[q], TY[q], TZ[q], NX[q], NY[q], NZ[q], A, B, C, AX[q], AY[q], AZ[q]);
                }
            } else {
                // some targets skip this sphere: compute the packs and keep only the wanted lanes
                for (int k = 0; k < n; ++k) {
                    const float4 A = sA[k], B = sB[k], C = sC[k];
#pragma unroll
                    for (int q = 0; q < NPK; ++q) {
                        float2 dx = f2(0.f, 0.f), dy = dx, dz = dx;
                        pair_x2<TRAC>(TX[q], TY[q], TZ[q], NX[q], NY[q], NZ[q], A, B, C, dx, dy, dz);
                        if (!sk[2 * q]) {
                            AX[q].x += dx.x;
                            AY[q].x += dy.x;
                            AZ[q].x += dz.x;
                        }
                        if (!sk[2 * q + 1]) {
                            AX[q].y += dx.y;
                            AY[q].y += dy.y;
                            AZ[q].y += dz.y;
                        }
                    }
                }
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
    float* out = partial + pr.poff + 3LL * mp * it.chunk;
#pragma unroll
    for (int q = 0; q < NPK; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = 2 * q + h;
            if (!val[u]) continue;
            float* o = out + 3LL * (it.t0 + threadIdx.x + u * kFarThreads - pr.p0);
            o[0] = h ? AX[q].y : AX[q].x;
            o[1] = h ? AY[q].y : AY[q].x;
            o[2] = h ? AZ[q].y : AZ[q].x;
        }
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
    __shared__ unsigned votes_buf[2][kFarThreads / 32];
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
    int parity = 0;
    for (int s = it.s0; s < it.s1; ++s, parity ^= 1) {
        bool sk[TPT];
        bool none = true;
        unsigned vote = 0;
#pragma unroll
        for (int u = 0; u < TPT; ++u) {
            sk[u] = !val[u] || excluded(g.nbr_src, cur[u], end[u], sid[u], s) || tgt_level(g, g.cs32, sid[u], s) >= 0;
            none = none && !sk[u];
            if (val[u]) vote |= sk[u] ? kBitSkip : level_bit(g, g.cs32, sid[u], s);
        }
        const unsigned votes = cta_or(vote, votes_buf, parity);
        if (!(votes & ~kBitSkip)) continue;  // every target skips this sphere
        const float4 *SP, *SF;
        int g0, gl;
        pick_sources(g, s, votes, src, SP, SF, g0, gl);
        for (int base = 0; base < gl; base += kFarTile32) {
            const int n = min(kFarTile32, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sp[k] = SP[g0 + base + k];
                sf[k] = SF[g0 + base + k];
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

// ---------------------------------------------------------------- several right-hand sides, one geometry
// The context holds nrep identical copies (replicas) of one problem, replica r in problem r with
// points [r*rep_M, (r+1)*rep_M). Work items are those of replica 0; blockIdx.y selects KB replicas.
// Per pair the geometry (r, 1/r, r^-5, r.n) is computed once and applied to the KB densities, so
// a pair-RHS costs 8 FP32 operations + 1 shared load instead of 20 + 2. Per RHS the arithmetic and
// the summation order are those of k_far32<TRAC, 1>, so every replica's sums equal bit for bit what
// the one-target-per-thread kernel gives for that density alone.
template <bool TRAC, int KB>
__global__ void __launch_bounds__(kFarThreads) k_far32_rep(DevGeom g, const FarItem* __restrict__ items, int nrep,
                                                          int rep_M, const float4* __restrict__ src,
                                                          float* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    const int r0 = blockIdx.y * KB;
    const int nr = min(KB, nrep - r0);
    bool any = g.active == nullptr;
    for (int r = 0; r < nr && !any; ++r) any = g.active[r0 + r] != 0;
    if (!any) return;
    __shared__ float4 sp[kRepTile];
    __shared__ float4 sf[KB][kRepTile];
    __shared__ unsigned votes_buf[2][kFarThreads / 32];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int t = it.t0 + threadIdx.x;
    const bool va = t < it.t1;
    const float4 tp = va ? g.pos32[t] : z4;
    const float4 tn = (TRAC && va) ? g.nrm32[t] : z4;
    const int sa = va ? __float_as_int(tp.w) : -1;
    int ca = va ? g.nbr_start[sa] : 0;
    const int ea = va ? g.nbr_start[sa + 1] : 0;
    float ax[KB], ay[KB], az[KB];
#pragma unroll
    for (int r = 0; r < KB; ++r) ax[r] = ay[r] = az[r] = 0.f;
    int parity = 0;
    for (int s = it.s0; s < it.s1; ++s, parity ^= 1) {
        const bool sk = !va || excluded(g.nbr_src, ca, ea, sa, s) || tgt_level(g, g.cs32, sa, s) >= 0;
        // the same per-CTA choice as k_far32<TRAC, 1> over the same targets (replica 0's items)
        const unsigned votes = cta_or(va ? (sk ? kBitSkip : level_bit(g, g.cs32, sa, s)) : 0u, votes_buf, parity);
        if (!(votes & ~kBitSkip)) continue;
        const float4 *SP, *SF;
        int g0, gl;
        const bool coarse = pick_sources(g, s, votes, src, SP, SF, g0, gl);
        const long long rstride = coarse ? (long long)g.cs32.crep : (long long)rep_M;  // replica r's sources
        for (int base = 0; base < gl; base += kRepTile) {
            const int n = min(kRepTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sp[k] = SP[g0 + base + k];
#pragma unroll
                for (int r = 0; r < KB; ++r) sf[r][k] = r < nr ? SF[(r0 + r) * rstride + g0 + base + k] : z4;
            }
            __syncthreads();
            if (sk) continue;
            for (int k = 0; k < n; ++k) {
                const float4 sq = sp[k];
                const float rx = tp.x - sq.x, ry = tp.y - sq.y, rz = tp.z - sq.z;
                const float r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                if (TRAC) {
                    const float ri5 = rpow5_mufu(r2);
                    const float rn = fmaf(rx, tn.x, fmaf(ry, tn.y, rz * tn.z));
#pragma unroll
                    for (int r = 0; r < KB; ++r) {
                        const float4 f = sf[r][k];
                        const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
                        const float kk = (rf * rn) * ri5;
                        ax[r] = fmaf(kk, rx, ax[r]);
                        ay[r] = fmaf(kk, ry, ay[r]);
                        az[r] = fmaf(kk, rz, az[r]);
                    }
                } else {
                    const float ri = rsqrt_mufu(r2), q = rcp_mufu(r2);
                    const float ri3 = q * ri;
#pragma unroll
                    for (int r = 0; r < KB; ++r) {
                        const float4 f = sf[r][k];
                        const float rf = fmaf(rx, f.x, fmaf(ry, f.y, rz * f.z));
                        const float kk = rf * ri3;
                        ax[r] = fmaf(f.x, ri, fmaf(kk, rx, ax[r]));
                        ay[r] = fmaf(f.y, ri, fmaf(kk, ry, ay[r]));
                        az[r] = fmaf(f.z, ri, fmaf(kk, rz, az[r]));
                    }
                }
            }
        }
    }
    if (!va) return;
#pragma unroll
    for (int r = 0; r < KB; ++r) {
        if (r < nr) {
            const Problem pr = g.problems[r0 + r];
            float* o = partial + pr.poff + 3LL * (pr.p1 - pr.p0) * it.chunk + 3LL * t;
            o[0] = ax[r];
            o[1] = ay[r];
            o[2] = az[r];
        }
    }
}

// ---------------------------------------------------------------- coarse targets (FP32)
// One CTA per work item: nodes [k0, k0 + nb) of an entry (target sphere t, level l, or its grid
// points for l = -1) against a range of its candidate source spheres, each resolved per geometry
// (k_ct_classify: counted only if tgt_level(t, s) == l, the host listing boundary cases under both
// levels; read from its coarse level for t, the nodes lying on t's surface, or its grid). The CTA's threads form
// 128 / w slices of w threads: thread (node, slice) takes every (128 / w)-th staged pair of source
// points, so small entries keep every thread busy. A thread's target sits duplicated in both FP32x2
// lanes and the sources are staged two to a pack, (x1,x2,y1,y2) (z1,z2,fx1,fx2) (fy1,fy2,fz1,fz2):
// one packed pair_x2 evaluates two pairs (a candidate with an odd count ends with a zero-strength
// point 1e18 away). Consecutive candidates share a staged tile until it holds kFarTile32 sources (a
// candidate larger than the room left continues in the next tile), so the many small coarse levels
// of an entry cost one pair of barriers per tile, not per candidate. The lanes' and slices' sums are
// added in a fixed order.
template <bool TRAC>
__global__ void __launch_bounds__(kFarThreads) k_far32_ct(DevGeom g, const CtWork* __restrict__ works,
                                                         const float4* __restrict__ src, float* __restrict__ partial) {
    const CtWork w = works[blockIdx.x];
    const CoarseSet& cs = g.cs32;
    const CtEnt e = cs.ctent[w.ent];
    if (g.active && !g.active[e.problem]) return;
    constexpr int kPk = kFarTile32 / 2;
    __shared__ float4 sA[kPk], sB[kPk], sC[kPk];
    __shared__ float red[3][kFarThreads];
    const int nslice = kFarThreads / w.w;
    const int node = threadIdx.x % w.w, slice = threadIdx.x / w.w;
    const bool val = node < w.nb;
    const int cn = e.q0 + w.k0 + node;
    const bool grid = e.l < 0;  // the sphere's grid points (CTA-uniform)
    // an empty slot sits 1e18 away: its terms are finite (and not written)
    const float4 P = val ? (grid ? g.pos32[cn] : cs.cpos32[cn]) : make_float4(1e18f, 1e18f, 1e18f, 0.f);
    const float4 Nn = (TRAC && val) ? (grid ? g.nrm32[cn] : cs.cnrm32[cn]) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 TX = f2(P.x, P.x), TY = f2(P.y, P.y), TZ = f2(P.z, P.z);
    const float2 NX = f2(Nn.x, Nn.x), NY = f2(Nn.y, Nn.y), NZ = f2(Nn.z, Nn.z);
    float2 AX = f2(0.f, 0.f), AY = AX, AZ = AX;
    // cursor over the candidates (CTA-uniform: every thread walks the same list): candidate i,
    // sources [off, ...) of it not staged yet
    int i = w.sa, off = 0;
    while (true) {
        __syncthreads();  // the previous tile has been read
        int np = 0;       // packs staged in this tile
        while (i < w.sb && np < kPk) {
            const int2 cc = cs.ctcand[i];
            if (cc.y == 0) {  // a boundary candidate of a neighbouring level
                ++i;
                continue;
            }
            const bool coarse = cc.y < 0;
            const float4* SP = coarse ? cs.cpos32 : g.pos32;
            const float4* SF = coarse ? cs.csrc : src;
            const int g0 = cc.x + off, gl = coarse ? -cc.y : cc.y;
            const int n = min(gl - off, 2 * (kPk - np));  // odd only at the candidate's end
            const int npk = (n + 1) >> 1;
            for (int k = threadIdx.x; k < npk; k += kFarThreads) {
                const int k1 = 2 * k, k2 = 2 * k + 1;
                const float4 p1 = SP[g0 + k1], f1 = SF[g0 + k1];
                const float4 p2 = k2 < n ? SP[g0 + k2] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
                const float4 q2 = k2 < n ? SF[g0 + k2] : make_float4(0.f, 0.f, 0.f, 0.f);
                sA[np + k] = make_float4(p1.x, p2.x, p1.y, p2.y);
                sB[np + k] = make_float4(p1.z, p2.z, f1.x, q2.x);
                sC[np + k] = make_float4(f1.y, q2.y, f1.z, q2.z);
            }
            np += npk;
            off += n;
            if (off >= gl) {
                ++i;
                off = 0;
            }
        }
        if (np == 0) break;
        __syncthreads();
#pragma unroll 4
        for (int k = slice; k < np; k += nslice)
            pair_x2<TRAC>(TX, TY, TZ, NX, NY, NZ, sA[k], sB[k], sC[k], AX, AY, AZ);
    }
    red[0][threadIdx.x] = AX.x + AX.y;
    red[1][threadIdx.x] = AY.x + AY.y;
    red[2][threadIdx.x] = AZ.x + AZ.y;
    __syncthreads();
    if (slice == 0 && val) {
        float x = 0.f, y = 0.f, z = 0.f;
        for (int sl = 0; sl < nslice; ++sl) {
            x += red[0][node + sl * w.w];
            y += red[1][node + sl * w.w];
            z += red[2][node + sl * w.w];
        }
        float* o = partial + e.poff + 3LL * ((long long)w.chunk * e.n + w.k0 + node);
        o[0] = x;
        o[1] = y;
        o[2] = z;
    }
}

// Per geometry: each entry's candidates resolved once. A candidate s of entry (t, l) counts if
// tgt_level(t, s) == l (the same rule for the listed and the grid entries, so every far pair lands in
// exactly one entry) and is read from its coarse level for t (level_bit) or its grid points.
__global__ void k_ct_classify(DevGeom g, CoarseSet cs) {
    const CtEnt e = cs.ctent[blockIdx.x];
    for (int i = threadIdx.x; i < e.nsrc; i += blockDim.x) {
        const int s = cs.ctsrc[e.src0 + i];
        int2 cc = make_int2(0, 0);
        if (tgt_level(g, cs, e.t, s) == e.l) {
            const unsigned b = level_bit(g, cs, e.t, s);
            if (b & kBitFine) {
                cc = make_int2(g.gidx[s], g.glen[s]);
            } else {
                const int4 L = cs.clev[s * kCoarseLevels + (31 - __clz(b))];
                cc = make_int2(L.y, -L.z);
            }
        }
        cs.ctcand[e.src0 + i] = cc;
    }
}

// the chunks' sums of every entry's nodes, in fixed order, into ctu (listed) or the grid slot (grid)
__global__ void k_ct_sum(DevGeom g, const float* __restrict__ partial) {
    const CoarseSet& cs = g.cs32;
    const CtEnt e = cs.ctent[blockIdx.x];
    if (g.active && !g.active[e.problem]) return;
    // CTA (entry, block of blockDim.x nodes)
    for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < e.n; k += blockDim.x * gridDim.y) {
        float x = 0.f, y = 0.f, z = 0.f;
        for (int c = 0; c < e.nchunks; ++c) {
            const float* o = partial + e.poff + 3LL * ((long long)c * e.n + k);
            x += o[0];
            y += o[1];
            z += o[2];
        }
        if (e.l >= 0) cs.ctu[e.q0 + k] = make_float4(x, y, z, 0.f);
        else {
            float* o = cs.ctinterp + 3LL * ((long long)kCoarseLevels * g.M + e.q0 + k);
            o[0] = x;
            o[1] = y;
            o[2] = z;
        }
    }
}

// Interpolation of the listed entries' node values to their spheres' grids: u(nu_j) = sum_k w_k
// K_pe(nu_j . nu_k) u_k (the transposed coarse map, exact for fields of degree <= pe on the sphere).
// A small GEMM per map (order p, level pe): CTA tile = 128 grid points x up to kCiEnt entries of that
// map; each map element read (coalesced, [node][grid point]) serves the entries' 3 components, whose
// node values are staged kCiK nodes at a time in shared memory. Two entries per tile: the map stays in
// L2 and more CTAs hide its latency (one CTA per SM with 8 entries on cfg2). Each entry's result goes
// to its level slot of ctinterp.
constexpr int kCiK = 32;  // entries per tile: kCiEnt; grid points per tile: kCiPts (one per thread)
static_assert(kCiPts == 128, "k_ct_interp runs one grid point per thread of 128");
__global__ void __launch_bounds__(128) k_ct_interp(DevGeom g) {
    const CoarseSet& cs = g.cs32;
    const CtITile d = cs.ctitile[blockIdx.x];
    __shared__ float4 U[kCiK][kCiEnt];
    __shared__ int eq0[kCiEnt], eon[kCiEnt];
    __shared__ long long ebase[kCiEnt];
    if (threadIdx.x < kCiEnt) {
        const int e = threadIdx.x;
        eon[e] = 0;
        eq0[e] = 0;
        ebase[e] = 0;
        if (e < d.ne) {
            const CtEnt en = cs.ctent[cs.ctient[d.e0 + e]];
            eon[e] = !g.active || g.active[en.problem];
            eq0[e] = en.q0;
            ebase[e] = (long long)en.l * g.M + g.gidx[en.t];
        }
    }
    __syncthreads();
    const int j = d.j0 + threadIdx.x;
    const bool val = j < d.ng;
    const float* MT = cs.cmapT + d.mapoff + (val ? j : 0);
    float acc[kCiEnt][3];
#pragma unroll
    for (int e = 0; e < kCiEnt; ++e) acc[e][0] = acc[e][1] = acc[e][2] = 0.f;
    for (int k0 = 0; k0 < d.n; k0 += kCiK) {
        const int nk = min(kCiK, d.n - k0);
        // the chunk's map column in registers first: kCiK independent loads in flight per thread
        float mk[kCiK];
#pragma unroll
        for (int kk = 0; kk < kCiK; ++kk) mk[kk] = (val && kk < nk) ? __ldg(MT + (long long)(k0 + kk) * d.ng) : 0.f;
        __syncthreads();
        for (int idx = threadIdx.x; idx < kCiK * kCiEnt; idx += 128) {
            const int kk = idx / kCiEnt, e = idx % kCiEnt;
            U[kk][e] = (kk < nk && eon[e]) ? cs.ctu[eq0[e] + k0 + kk] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        // rows past nk hold zeros in both operands
#pragma unroll
        for (int kk = 0; kk < kCiK; ++kk) {
            const float m = mk[kk];
#pragma unroll
            for (int e = 0; e < kCiEnt; ++e) {
                const float4 u = U[kk][e];
                acc[e][0] = fmaf(m, u.x, acc[e][0]);
                acc[e][1] = fmaf(m, u.y, acc[e][1]);
                acc[e][2] = fmaf(m, u.z, acc[e][2]);
            }
        }
    }
    if (!val) return;
#pragma unroll
    for (int e = 0; e < kCiEnt; ++e) {
        if (e >= d.ne || !eon[e]) continue;
        float* o = cs.ctinterp + 3LL * (ebase[e] + j);
        o[0] = acc[e][0];
        o[1] = acc[e][1];
        o[2] = acc[e][2];
    }
}

// The interpolation on the tcgen05 tensor cores (FP32 set): per map the GEMM
//   D [128 grid points x 48] = A [128 x N_e] . B [48 x N_e]^T,
// A = the map [grid point][coarse node] (pre-split to 3xTF32 and tiled once per geometry, cmapI), B =
// the coarse-node field of 16 entries, one row per (entry, component), gathered from ctu and split by
// the threads; K runs over the coarse nodes in chunks of 32. One thread issues each chunk's 12 MMAs
// and waits (bounded); even and odd chunks accumulate in two tensor-memory tiles (columns 0-47 and
// 64-111), which halves each accumulation chain, and the two are added in FP32 at the end. Each thread
// then writes its grid point's values of the 16 entries to their level slots of ctinterp. Every D
// element is the same sum whichever entries share the tile.
__global__ void __launch_bounds__(128) k_ct_interp_tc(DevGeom g) {
    const CoarseSet& cs = g.cs32;
    const CtITile d = cs.ctitile_tc[blockIdx.x];
    extern __shared__ __align__(1024) unsigned char ci_smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ int s_fail;
    __shared__ int eq0[kCsTcSph];
    __shared__ long long ebase[kCsTcSph];
    __shared__ unsigned char eon[kCsTcSph];
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid < kCsTcSph) {
        eon[tid] = 0;
        eq0[tid] = 0;
        ebase[tid] = 0;
        if (tid < d.ne) {
            const CtEnt en = cs.ctent[cs.ctient_tc[d.e0 + tid]];
            eon[tid] = (!g.active || g.active[en.problem]) ? 1 : 0;
            eq0[tid] = en.q0;
            ebase[tid] = (long long)en.l * g.M + g.gidx[en.t];
        }
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_fence_init();
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    constexpr uint32_t idesc = tc::idesc_tf32(128, kCsTcN);
    unsigned char* sAh = ci_smem;
    unsigned char* sAl = ci_smem + kCsTcABytes;
    unsigned char* sBh = ci_smem + 2 * kCsTcABytes;
    unsigned char* sBl = sBh + kCsTcBBytes;
    const int j = d.j0 + tid;  // this thread's D row (grid point)
    const bool rvalid = j < d.ng;
    const int nck = (d.n + kCsTcK - 1) / kCsTcK;
    const float4* __restrict__ At = cs.cmapI + ((long long)d.mapoff + (long long)(d.j0 / 128) * nck * 2 * 128 * kCsTcK) / 4;
    unsigned phase = 0;
    bool failed = false;
    for (int ch = 0; ch < nck; ++ch) {
        const int k0 = ch * kCsTcK;
        {
            const float4* src_h = At + (long long)ch * 2 * (kCsTcABytes / 16);
            const float4* src_l = src_h + kCsTcABytes / 16;
#pragma unroll
            for (int v = tid; v < kCsTcABytes / 16; v += 128) {
                reinterpret_cast<float4*>(sAh)[v] = __ldg(src_h + v);
                reinterpret_cast<float4*>(sAl)[v] = __ldg(src_l + v);
            }
        }
        for (int v = tid; v < kCsTcSph * kCsTcK; v += 128) {
            const int e = v / kCsTcK, kk = v % kCsTcK, k = k0 + kk;
            const float4 u = (e < d.ne && eon[e] && k < d.n) ? cs.ctu[eq0[e] + k] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float uc[3] = {u.x, u.y, u.z};
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const float h = tc::tf32_hi(uc[cc]), l = tc::tf32_hi(uc[cc] - h);
                const uint32_t off = tc::kmajor_offset(3 * e + cc, kk, kCsTcK);
                *reinterpret_cast<float*>(sBh + off) = h;
                *reinterpret_cast<float*>(sBl + off) = l;
            }
        }
        tc::fence_smem_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t ah0 = tc::smem_u32(sAh), al0 = tc::smem_u32(sAl);
            const uint32_t bh0 = tc::smem_u32(sBh), bl0 = tc::smem_u32(sBl);
            constexpr uint32_t sbo = (kCsTcK / 4) * 128;
#pragma unroll
            for (int ks = 0; ks < kCsTcK / 8; ++ks) {
                const uint32_t o = ks * 256;
                const uint64_t ah = tc::sdesc(ah0 + o, 128, sbo), al = tc::sdesc(al0 + o, 128, sbo);
                const uint64_t bh = tc::sdesc(bh0 + o, 128, sbo), bl = tc::sdesc(bl0 + o, 128, sbo);
                const uint32_t dt = tmem + 64 * (ch & 1);
                tc::mma_tf32(dt, ah, bh, idesc, ch > 1 || ks > 0);
                tc::mma_tf32(dt, ah, bl, idesc, true);
                tc::mma_tf32(dt, al, bh, idesc, true);
            }
            tc::mma_commit(&mbar);
            if (!tc::mbar_wait_bounded(&mbar, phase, kCsTcWaitPolls)) s_fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        if (s_fail) {
            failed = true;
            break;
        }
    }
    if (!failed && nck > 0) {
        tc::fence_after_sync();
        float da[32], db[32];
        const uint32_t lane_base = uint32_t(warp * 32) << 16;
        tc::tmem_ld_32x32b_x32(tmem + lane_base, da);       // even chunks, columns 0-31
        tc::tmem_ld_32x32b_x32(tmem + 32 + lane_base, db);  // columns 32-63 (48-63 unused)
        if (nck > 1) {  // odd chunks
            float ea[32], eb[32];
            tc::tmem_ld_32x32b_x32(tmem + 64 + lane_base, ea);
            tc::tmem_ld_32x32b_x32(tmem + 96 + lane_base, eb);
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                da[q] += ea[q];
                db[q] += eb[q];
            }
        }
        if (rvalid) {
#pragma unroll
            for (int e = 0; e < kCsTcSph; ++e) {
                if (e >= d.ne || !eon[e]) continue;
                float* o = cs.ctinterp + 3LL * (ebase[e] + j);
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) {
                    const int col = 3 * e + cc;
                    o[cc] = col < 32 ? da[col] : db[col - 32];
                }
            }
        }
    } else if (failed && tid == 0 && g.err) {
        atomicExch(g.err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 128);
    }
}

template <bool TRAC>
__global__ void __launch_bounds__(kFarThreads) k_far64(DevGeom g, const FarItem* __restrict__ items,
                                                      const double4_32a* __restrict__ src, double* __restrict__ partial) {
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ double4_32a sp[kFarTile];
    __shared__ double4_32a sf[kFarTile];
    const int ta = it.t0 + threadIdx.x;
    const bool va = ta < it.t1;
    const double4_32a z4 = make_double4_32a(0, 0, 0, 0);
    const double4_32a pa = va ? g.pos64[ta] : z4;
    const double4_32a na = (TRAC && va) ? g.nrm64[ta] : z4;
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
// FP64. Used for the high-precision passes of the mixed-precision solve. Two targets share a
// thread as the two lanes of packed FP32x2 instructions (FFMA2/FADD2/FMUL2): every instruction
// advances two pairs, which halves the issue slots the error-free transformations take.
// The _rn intrinsics keep every rounding explicit: the compiler may not contract a product into a
// later addition, which would break the error-free transformations below.
// (float-float primitives and the dfv type: df.h)
// packed float-float accumulators of two targets: traction (or the single layer for KIND 0) and, for
// KIND 2, the single layer
struct DfAcc {
    float2 xh, xl, yh, yl, zh, zl;
    float2 sxh, sxl, syh, syl, szh, szl;
};

// one source (qh + ql, strength fh + fl) against the two packed targets (mx, my, mz) with normals
// (n0, n1, n2); masked: keep scales the source weight per lane
template <int KIND>
__device__ __forceinline__ void df_pair(const df2& mx, const df2& my, const df2& mz, const df2& n0, const df2& n1,
                                        const df2& n2, const float4& qh, const float4& ql, const float4& fh,
                                        const float4& fl, bool masked, float2 keep, DfAcc& a) {
    constexpr bool TRAC = KIND != 0, SL = KIND != 1;
    const df2 dx = two_sum(mx.h, f2(-qh.x, -qh.x));
    const df2 dy = two_sum(my.h, f2(-qh.y, -qh.y));
    const df2 dz = two_sum(mz.h, f2(-qh.z, -qh.z));
    const df2 rx{dx.h, __fadd2_rn(dx.l, __fadd2_rn(mx.l, f2(-ql.x, -ql.x)))};
    const df2 ry{dy.h, __fadd2_rn(dy.l, __fadd2_rn(my.l, f2(-ql.y, -ql.y)))};
    const df2 rz{dz.h, __fadd2_rn(dz.l, __fadd2_rn(mz.l, f2(-ql.z, -ql.z)))};
    df2 f0{f2(fh.x, fh.x), f2(fl.x, fl.x)}, f1{f2(fh.y, fh.y), f2(fl.y, fl.y)}, fz{f2(fh.z, fh.z), f2(fl.z, fl.z)};
    if (masked) {
        f0 = {__fmul2_rn(f0.h, keep), __fmul2_rn(f0.l, keep)};
        f1 = {__fmul2_rn(f1.h, keep), __fmul2_rn(f1.l, keep)};
        fz = {__fmul2_rn(fz.h, keep), __fmul2_rn(fz.l, keep)};
    }
    const df2 r2 = df_sqr3(rx, ry, rz);
    const df2 ri = df_rsqrt(r2);
    const df2 rf = df_dot3(rx, f0, ry, f1, rz, fz);
    const df2 ri2 = df_mul_u(ri, ri);
    const df2 ri3 = df_mul_u(ri2, ri);
    if (TRAC) {  // (r.f)(r.n) r / r^5
        const df2 rn = df_dot3(rx, n0, ry, n1, rz, n2);
        const df2 k5 = df_mul_u(df_mul_u(rf, rn), df_mul_u(ri3, ri2));
        df_acc(a.xh, a.xl, df_mul_u(k5, rx));
        df_acc(a.yh, a.yl, df_mul_u(k5, ry));
        df_acc(a.zh, a.zl, df_mul_u(k5, rz));
    }
    if (SL) {  // f / r + (r.f) r / r^3
        const df2 k3 = df_mul_u(rf, ri3);
        float2& ah = KIND == 2 ? a.sxh : a.xh;
        float2& al = KIND == 2 ? a.sxl : a.xl;
        float2& bh = KIND == 2 ? a.syh : a.yh;
        float2& bl = KIND == 2 ? a.syl : a.yl;
        float2& ch = KIND == 2 ? a.szh : a.zh;
        float2& cl = KIND == 2 ? a.szl : a.zl;
        df_acc(ah, al, df_mul_u(f0, ri));
        df_acc(ah, al, df_mul_u(k3, rx));
        df_acc(bh, bl, df_mul_u(f1, ri));
        df_acc(bh, bl, df_mul_u(k3, ry));
        df_acc(ch, cl, df_mul_u(fz, ri));
        df_acc(ch, cl, df_mul_u(k3, rz));
    }
}

// KIND: 0 single layer -> partial; 1 traction -> partial; 2 both from the same sources in one pass
// (traction -> partial, single layer -> partial_sl), sharing r, 1/r and r.f between the two kernels.
template <int KIND>
__global__ void __launch_bounds__(kFarThreadsDF, 384 / kFarThreadsDF)
    k_far_dfx2(DevGeom g, const FarItem* __restrict__ items, const float4* __restrict__ src,
               double* __restrict__ partial, double* __restrict__ partial_sl) {
    constexpr bool TRAC = KIND != 0;
    constexpr int NT = kFarThreadsDF;
    const FarItem it = items[blockIdx.x];
    if (g.active && !g.active[it.problem]) return;
    __shared__ float4 sph[kFarTile], spl[kFarTile], sfh[kFarTile], sfl[kFarTile];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 PH[2], PL[2], NH[2], NL[2];
    int sid[2], cur[2], end[2];
    bool val[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int t = it.t0 + threadIdx.x + h * NT;
        val[h] = t < it.t1;
        PH[h] = val[h] ? g.pos32[t] : z4;
        PL[h] = val[h] ? g.pos32lo[t] : z4;
        NH[h] = (TRAC && val[h]) ? g.nrm32[t] : z4;
        NL[h] = (TRAC && val[h]) ? g.nrm32lo[t] : z4;
        sid[h] = val[h] ? __float_as_int(PH[h].w) : -1;
        cur[h] = val[h] ? g.nbr_start[sid[h]] : 0;
        end[h] = val[h] ? g.nbr_start[sid[h] + 1] : 0;
    }
    const df2 tx{f2(PH[0].x, PH[1].x), f2(PL[0].x, PL[1].x)}, ty{f2(PH[0].y, PH[1].y), f2(PL[0].y, PL[1].y)},
        tz{f2(PH[0].z, PH[1].z), f2(PL[0].z, PL[1].z)};
    const df2 n0{f2(NH[0].x, NH[1].x), f2(NL[0].x, NL[1].x)}, n1{f2(NH[0].y, NH[1].y), f2(NL[0].y, NL[1].y)},
        n2{f2(NH[0].z, NH[1].z), f2(NL[0].z, NL[1].z)};
    DfAcc acc;
    acc.xh = acc.xl = acc.yh = acc.yl = acc.zh = acc.zl = f2(0.f, 0.f);
    acc.sxh = acc.sxl = acc.syh = acc.syl = acc.szh = acc.szl = f2(0.f, 0.f);
    __shared__ unsigned votes_buf[2][NT / 32];
    auto pair = [&](const df2& mx, const df2& my, const df2& mz, const float4& qh, const float4& ql,
                    const float4& fh, const float4& fl, bool masked, float2 keep) {
        df_pair<KIND>(mx, my, mz, n0, n1, n2, qh, ql, fh, fl, masked, keep, acc);
    };
    int parity = 0;
    for (int s = it.s0; s < it.s1; ++s, parity ^= 1) {
        bool sk[2];
        sk[0] = !val[0] || excluded(g.nbr_src, cur[0], end[0], sid[0], s);
        sk[1] = !val[1] || excluded(g.nbr_src, cur[1], end[1], sid[1], s);
        unsigned vote = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (val[h]) vote |= sk[h] ? kBitSkip : level_bit(g, g.cshp, sid[h], s);
        const unsigned votes = cta_or<NT>(vote, votes_buf, parity);
        if (!(votes & ~kBitSkip)) continue;  // every target skips this sphere
        // coarse level of the float-float set, or the grid sources
        const bool coarse = !(votes & (kBitSkip | kBitFine));
        const float4 *QH = g.pos32, *QL = g.pos32lo, *QF = src;
        int g0 = g.gidx[s], gl = g.glen[s];
        if (coarse) {
            const int4 L = g.cshp.clev[s * kCoarseLevels + (31 - __clz(votes))];
            QH = g.cshp.cpos32;
            QL = g.cshp.cpos32lo;
            QF = g.cshp.csrc;
            g0 = L.y;
            gl = L.z;
        }
        const bool masked = sk[0] || sk[1];
        // A lane whose target skips this sphere is moved to a point 1e18 away and its source weight
        // is zeroed: its terms are exact zeros (r^-5 underflows, no 0*inf at r = 0 on its own sphere).
        const float2 keep = f2(sk[0] ? 0.f : 1.f, sk[1] ? 0.f : 1.f);
        const float2 far2 = f2(sk[0] ? 1e18f : 0.f, sk[1] ? 1e18f : 0.f);
        const df2 mx{__fadd2_rn(tx.h, far2), __fmul2_rn(tx.l, keep)};
        const df2 my{__fadd2_rn(ty.h, far2), __fmul2_rn(ty.l, keep)};
        const df2 mz{__fadd2_rn(tz.h, far2), __fmul2_rn(tz.l, keep)};
        for (int base = 0; base < gl; base += kFarTile) {
            const int n = min(kFarTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += NT) {
                sph[k] = QH[g0 + base + k];
                spl[k] = QL[g0 + base + k];
                sfh[k] = QF[2 * (g0 + base + k)];
                sfl[k] = QF[2 * (g0 + base + k) + 1];
            }
            __syncthreads();
            if (!masked) {
                for (int k = 0; k < n; ++k) pair(tx, ty, tz, sph[k], spl[k], sfh[k], sfl[k], false, keep);
            } else {
                for (int k = 0; k < n; ++k) pair(mx, my, mz, sph[k], spl[k], sfh[k], sfl[k], true, keep);
            }
        }
    }
    const Problem pr = g.problems[it.problem];
    const long long mp = pr.p1 - pr.p0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (!val[h]) continue;
        const long long off = pr.poff + 3LL * mp * it.chunk + 3LL * (it.t0 + threadIdx.x + h * NT - pr.p0);
        double* o = partial + off;
        o[0] = h ? double(acc.xh.y) + double(acc.xl.y) : double(acc.xh.x) + double(acc.xl.x);
        o[1] = h ? double(acc.yh.y) + double(acc.yl.y) : double(acc.yh.x) + double(acc.yl.x);
        o[2] = h ? double(acc.zh.y) + double(acc.zl.y) : double(acc.zh.x) + double(acc.zl.x);
        if (KIND == 2) {
            double* q = partial_sl + off;
            q[0] = h ? double(acc.sxh.y) + double(acc.sxl.y) : double(acc.sxh.x) + double(acc.sxl.x);
            q[1] = h ? double(acc.syh.y) + double(acc.syl.y) : double(acc.syh.x) + double(acc.syl.x);
            q[2] = h ? double(acc.szh.y) + double(acc.szl.y) : double(acc.szh.x) + double(acc.szl.x);
        }
    }
}

// The fused float-float pass with the float-float set's coarse targets: one CTA of kFarThreadsDF
// threads per work item, nodes [k0, k0 + nb) of an entry (coarse nodes of level l, or the sphere's
// grid points for l = -1), against the entry's candidates as k_ct_classify resolved them (float-float
// coarse level or grid). A block of w nodes (w = 64, 32, ..., 4) runs as w / 2 threads holding two
// nodes each, the packed lanes of df_pair, times 64 / w slices: slice i takes every (64 / w)-th staged
// source, and the slices' float-float sums are added in slice order. So an entry's last few nodes
// cost a fraction of a CTA, not a whole 64-node one. Partial sums [chunk][node][6] (traction, single
// layer).
__global__ void __launch_bounds__(kFarThreadsDF, 384 / kFarThreadsDF)
    k_far_df_ct(DevGeom g, const CtWork* __restrict__ works, const float4* __restrict__ src,
                double* __restrict__ partial) {
    constexpr int NT = kFarThreadsDF;
    const CtWork w = works[blockIdx.x];
    const CoarseSet& cs = g.cshp;
    const CtEnt e = cs.ctent[w.ent];
    if (g.active && !g.active[e.problem]) return;
    __shared__ float4 sph[kFarTile], spl[kFarTile], sfh[kFarTile], sfl[kFarTile];
    const bool grid = e.l < 0;  // CTA-uniform
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int hw = w.w >> 1, nslice = NT / hw;  // threads per slice, slices
    const int j = threadIdx.x % hw, slice = threadIdx.x / hw;
    float4 PH[2], PL[2], NH[2], NL[2];
    bool val[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int node = j + h * hw;
        val[h] = node < w.nb;
        const int cn = e.q0 + w.k0 + node;
        // an empty slot sits 1e18 away: its terms are finite (and not written)
        PH[h] = val[h] ? (grid ? g.pos32[cn] : cs.cpos32[cn]) : make_float4(1e18f, 1e18f, 1e18f, 0.f);
        PL[h] = val[h] ? (grid ? g.pos32lo[cn] : cs.cpos32lo[cn]) : z4;
        NH[h] = val[h] ? (grid ? g.nrm32[cn] : cs.cnrm32[cn]) : z4;
        NL[h] = val[h] ? (grid ? g.nrm32lo[cn] : cs.cnrm32lo[cn]) : z4;
    }
    const df2 tx{f2(PH[0].x, PH[1].x), f2(PL[0].x, PL[1].x)}, ty{f2(PH[0].y, PH[1].y), f2(PL[0].y, PL[1].y)},
        tz{f2(PH[0].z, PH[1].z), f2(PL[0].z, PL[1].z)};
    const df2 n0{f2(NH[0].x, NH[1].x), f2(NL[0].x, NL[1].x)}, n1{f2(NH[0].y, NH[1].y), f2(NL[0].y, NL[1].y)},
        n2{f2(NH[0].z, NH[1].z), f2(NL[0].z, NL[1].z)};
    DfAcc acc;
    acc.xh = acc.xl = acc.yh = acc.yl = acc.zh = acc.zl = f2(0.f, 0.f);
    acc.sxh = acc.sxl = acc.syh = acc.syl = acc.szh = acc.szl = f2(0.f, 0.f);
    const float2 one = f2(1.f, 1.f);
    __shared__ float2 red[12][NT];
    for (int i = w.sa; i < w.sb; ++i) {
        const int2 cc = cs.ctcand[i];  // CTA-uniform
        if (cc.y == 0) continue;       // a boundary candidate of a neighbouring level
        const bool coarse = cc.y < 0;
        const float4* QH = coarse ? cs.cpos32 : g.pos32;
        const float4* QL = coarse ? cs.cpos32lo : g.pos32lo;
        const float4* QF = coarse ? cs.csrc : src;
        const int g0 = cc.x, gl = coarse ? -cc.y : cc.y;
        for (int base = 0; base < gl; base += kFarTile) {
            const int n = min(kFarTile, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += NT) {
                sph[k] = QH[g0 + base + k];
                spl[k] = QL[g0 + base + k];
                sfh[k] = QF[2 * (g0 + base + k)];
                sfl[k] = QF[2 * (g0 + base + k) + 1];
            }
            __syncthreads();
            for (int k = slice; k < n; k += nslice)
                df_pair<2>(tx, ty, tz, n0, n1, n2, sph[k], spl[k], sfh[k], sfl[k], false, one, acc);
        }
    }
    if (nslice > 1) {  // CTA-uniform
        red[0][threadIdx.x] = acc.xh, red[1][threadIdx.x] = acc.xl;
        red[2][threadIdx.x] = acc.yh, red[3][threadIdx.x] = acc.yl;
        red[4][threadIdx.x] = acc.zh, red[5][threadIdx.x] = acc.zl;
        red[6][threadIdx.x] = acc.sxh, red[7][threadIdx.x] = acc.sxl;
        red[8][threadIdx.x] = acc.syh, red[9][threadIdx.x] = acc.syl;
        red[10][threadIdx.x] = acc.szh, red[11][threadIdx.x] = acc.szl;
        __syncthreads();
        if (slice != 0) return;
        for (int sl = 1; sl < nslice; ++sl) {
            const int t = j + sl * hw;
            df_acc(acc.xh, acc.xl, df2{red[0][t], red[1][t]});
            df_acc(acc.yh, acc.yl, df2{red[2][t], red[3][t]});
            df_acc(acc.zh, acc.zl, df2{red[4][t], red[5][t]});
            df_acc(acc.sxh, acc.sxl, df2{red[6][t], red[7][t]});
            df_acc(acc.syh, acc.syl, df2{red[8][t], red[9][t]});
            df_acc(acc.szh, acc.szl, df2{red[10][t], red[11][t]});
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (!val[h]) continue;
        double* o = partial + e.poff + 6LL * ((long long)w.chunk * e.n + w.k0 + j + h * hw);
        o[0] = h ? double(acc.xh.y) + double(acc.xl.y) : double(acc.xh.x) + double(acc.xl.x);
        o[1] = h ? double(acc.yh.y) + double(acc.yl.y) : double(acc.yh.x) + double(acc.yl.x);
        o[2] = h ? double(acc.zh.y) + double(acc.zl.y) : double(acc.zh.x) + double(acc.zl.x);
        o[3] = h ? double(acc.sxh.y) + double(acc.sxl.y) : double(acc.sxh.x) + double(acc.sxl.x);
        o[4] = h ? double(acc.syh.y) + double(acc.syl.y) : double(acc.syh.x) + double(acc.syl.x);
        o[5] = h ? double(acc.szh.y) + double(acc.szl.y) : double(acc.szh.x) + double(acc.szl.x);
    }
}

// the chunks' sums of every float-float entry's nodes, in fixed order, into ctud (listed) or the grid
// slot of ctinterpd (grid entries)
__global__ void k_ct_sum_df(DevGeom g, const double* __restrict__ partial) {
    const CoarseSet& cs = g.cshp;
    const CtEnt e = cs.ctent[blockIdx.x];
    if (g.active && !g.active[e.problem]) return;
    // CTA (entry, block of blockDim.x nodes)
    for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < e.n; k += blockDim.x * gridDim.y) {
        double v[6] = {0, 0, 0, 0, 0, 0};
        for (int c = 0; c < e.nchunks; ++c) {
            const double* o = partial + e.poff + 6LL * ((long long)c * e.n + k);
#pragma unroll
            for (int q = 0; q < 6; ++q) v[q] += o[q];
        }
        double* d = e.l >= 0 ? cs.ctud + 6LL * (e.q0 + k) : cs.ctinterpd + 6LL * ((long long)kCoarseLevels * g.M + e.q0 + k);
#pragma unroll
        for (int q = 0; q < 6; ++q) d[q] = v[q];
    }
}

// The float-float set's interpolation in float-float arithmetic on the FP32 pipes (the FP64 pipe is
// 1/58 of them): maps stored as (hi, lo) float pairs, the entries' node values split into (hi, lo) in
// shared memory, products by df_mul_u and sums by df_acc (~2^-44 relative to the sum of |terms|).
// CTA tile: 256 grid points (two per thread, the packed lanes) x kCiEntD entries x 6 components.
constexpr int kCiKD = 8;  // kCiEntD = 1 entry per tile: 2x the CTAs of two (177 on cfg2, 152 SMs)
static_assert(kCiPtsD == 2 * 128, "k_ct_interp_df runs two grid points per thread of 128");
__global__ void __launch_bounds__(128) k_ct_interp_df(DevGeom g) {
    const CoarseSet& cs = g.cshp;
    const CtITile d = cs.ctitile[blockIdx.x];
    __shared__ float2 U[kCiKD][kCiEntD][6];
    __shared__ int eq0[kCiEntD], eon[kCiEntD];
    __shared__ long long ebase[kCiEntD];
    if (threadIdx.x < kCiEntD) {
        const int e = threadIdx.x;
        eon[e] = 0;
        eq0[e] = 0;
        ebase[e] = 0;
        if (e < d.ne) {
            const CtEnt en = cs.ctent[cs.ctient[d.e0 + e]];
            eon[e] = !g.active || g.active[en.problem];
            eq0[e] = en.q0;
            ebase[e] = (long long)en.l * g.M + g.gidx[en.t];
        }
    }
    __syncthreads();
    // grid points j, j + 1 (ng is even, so both or neither exist); (hi, lo) pairs of both in one float4
    const int j = d.j0 + 2 * threadIdx.x;
    const bool val = j < d.ng;
    const float4* MT = reinterpret_cast<const float4*>(cs.cmapTdf + d.mapoff + (val ? j : 0));
    const long long row = d.ng / 2;  // float4 per map row
    float2 ah[kCiEntD][6], al[kCiEntD][6];
#pragma unroll
    for (int e = 0; e < kCiEntD; ++e)
#pragma unroll
        for (int q = 0; q < 6; ++q) ah[e][q] = al[e][q] = f2(0.f, 0.f);
    for (int k0 = 0; k0 < d.n; k0 += kCiKD) {
        const int nk = min(kCiKD, d.n - k0);
        float4 mk[kCiKD];
#pragma unroll
        for (int kk = 0; kk < kCiKD; ++kk)
            mk[kk] = (val && kk < nk) ? __ldg(MT + (long long)(k0 + kk) * row) : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        for (int idx = threadIdx.x; idx < kCiKD * kCiEntD * 6; idx += 128) {
            const int q = idx % 6, e = (idx / 6) % kCiEntD, kk = idx / (6 * kCiEntD);
            const double u = (kk < nk && eon[e]) ? cs.ctud[6LL * (eq0[e] + k0 + kk) + q] : 0.0;
            const float h = float(u);
            U[kk][e][q] = f2(h, float(u - double(h)));
        }
        __syncthreads();
        // rows past nk hold zeros in both operands
#pragma unroll
        for (int kk = 0; kk < kCiKD; ++kk) {
            const df2 m{f2(mk[kk].x, mk[kk].z), f2(mk[kk].y, mk[kk].w)};
#pragma unroll
            for (int e = 0; e < kCiEntD; ++e)
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const float2 u = U[kk][e][q];
                    df_acc(ah[e][q], al[e][q], df_mul_u(m, df2{f2(u.x, u.x), f2(u.y, u.y)}));
                }
        }
    }
    if (!val) return;
#pragma unroll
    for (int e = 0; e < kCiEntD; ++e) {
        if (e >= d.ne || !eon[e]) continue;
        double* o = cs.ctinterpd + 6LL * (ebase[e] + j);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            o[q] = double(ah[e][q].x) + double(al[e][q].x);
            o[6 + q] = double(ah[e][q].y) + double(al[e][q].y);
        }
    }
}

// Float-float traction and single layer (the fused high-precision pass) for nrep replicas of one
// problem (see k_far32_rep): one target per thread, replica 0's work items, KB columns per CTA.
// The pair geometry (r, r^2, 1/r, r^-3, r^-5, r.n) is evaluated once and serves the KB columns;
// per column the arithmetic and the source order are those of k_far_dfx2<2>, so each column's
// sums equal bit for bit the single-problem pass on that column.
template <int KB>
__global__ void __launch_bounds__(kFarThreads) k_far_df_rep(DevGeom g, const FarItem* __restrict__ items, int nrep,
                                                           int rep_M, const float4* __restrict__ src,
                                                           double* __restrict__ partial,
                                                           double* __restrict__ partial_sl) {
    const FarItem it = items[blockIdx.x];
    const int r0 = blockIdx.y * KB;
    const int nr = min(KB, nrep - r0);
    bool any = g.active == nullptr;
    for (int r = 0; r < nr && !any; ++r) any = g.active[r0 + r] != 0;
    if (!any) return;
    __shared__ float4 sph[kRepTileDF], spl[kRepTileDF];
    __shared__ float4 sfh[KB][kRepTileDF], sfl[KB][kRepTileDF];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int t = it.t0 + threadIdx.x;
    const bool va = t < it.t1;
    const float4 PH = va ? g.pos32[t] : z4, PL = va ? g.pos32lo[t] : z4;
    const float4 NH = va ? g.nrm32[t] : z4, NL = va ? g.nrm32lo[t] : z4;
    const int sa = va ? __float_as_int(PH.w) : -1;
    int ca = va ? g.nbr_start[sa] : 0;
    const int ea = va ? g.nbr_start[sa + 1] : 0;
    const df1 n0{NH.x, NL.x}, n1{NH.y, NL.y}, n2{NH.z, NL.z};
    float th[KB][3], tl[KB][3], sh[KB][3], sl[KB][3];
#pragma unroll
    for (int r = 0; r < KB; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) th[r][d] = tl[r][d] = sh[r][d] = sl[r][d] = 0.f;
    for (int s = it.s0; s < it.s1; ++s) {
        const bool sk = !va || excluded(g.nbr_src, ca, ea, sa, s);
        if (__syncthreads_and(sk)) continue;
        const int g0 = g.gidx[s], gl = g.glen[s];
        for (int base = 0; base < gl; base += kRepTileDF) {
            const int n = min(kRepTileDF, gl - base);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += kFarThreads) {
                sph[k] = g.pos32[g0 + base + k];
                spl[k] = g.pos32lo[g0 + base + k];
#pragma unroll
                for (int r = 0; r < KB; ++r) {
                    const long long i = (long long)(r0 + r) * rep_M + g0 + base + k;
                    sfh[r][k] = r < nr ? src[2 * i] : z4;
                    sfl[r][k] = r < nr ? src[2 * i + 1] : z4;
                }
            }
            __syncthreads();
            if (sk) continue;
            for (int k = 0; k < n; ++k) {
                const float4 qh = sph[k], ql = spl[k];
                const df1 dx = two_sum(PH.x, -qh.x), dy = two_sum(PH.y, -qh.y), dz = two_sum(PH.z, -qh.z);
                const df1 rx{dx.h, v_add(dx.l, v_add(PL.x, -ql.x))};
                const df1 ry{dy.h, v_add(dy.l, v_add(PL.y, -ql.y))};
                const df1 rz{dz.h, v_add(dz.l, v_add(PL.z, -ql.z))};
                const df1 ri = df_rsqrt(df_sqr3(rx, ry, rz));
                const df1 ri2 = df_mul_u(ri, ri);
                const df1 ri3 = df_mul_u(ri2, ri);
                const df1 rn = df_dot3(rx, n0, ry, n1, rz, n2);
                const df1 ri5 = df_mul_u(ri3, ri2);
#pragma unroll
                for (int r = 0; r < KB; ++r) {
                    const float4 fh = sfh[r][k], fl = sfl[r][k];
                    const df1 f0{fh.x, fl.x}, f1{fh.y, fl.y}, fz{fh.z, fl.z};
                    const df1 rf = df_dot3(rx, f0, ry, f1, rz, fz);
                    const df1 k5 = df_mul_u(df_mul_u(rf, rn), ri5);
                    df_acc(th[r][0], tl[r][0], df_mul_u(k5, rx));
                    df_acc(th[r][1], tl[r][1], df_mul_u(k5, ry));
                    df_acc(th[r][2], tl[r][2], df_mul_u(k5, rz));
                    const df1 k3 = df_mul_u(rf, ri3);
                    df_acc(sh[r][0], sl[r][0], df_mul_u(f0, ri));
                    df_acc(sh[r][0], sl[r][0], df_mul_u(k3, rx));
                    df_acc(sh[r][1], sl[r][1], df_mul_u(f1, ri));
                    df_acc(sh[r][1], sl[r][1], df_mul_u(k3, ry));
                    df_acc(sh[r][2], sl[r][2], df_mul_u(fz, ri));
                    df_acc(sh[r][2], sl[r][2], df_mul_u(k3, rz));
                }
            }
        }
    }
    if (!va) return;
#pragma unroll
    for (int r = 0; r < KB; ++r) {
        if (r < nr) {
            const Problem pr = g.problems[r0 + r];
            const long long off = pr.poff + 3LL * (pr.p1 - pr.p0) * it.chunk + 3LL * t;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                partial[off + d] = double(th[r][d]) + double(tl[r][d]);
                partial_sl[off + d] = double(sh[r][d]) + double(sl[r][d]);
            }
        }
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
                           double4_32a* __restrict__ s64) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    if (g.active && !g.active[g.prob[g.sid[i]]]) return;
    const double w = g.weights[i] * c;
    const double fx = x[3 * i] * w, fy = x[3 * i + 1] * w, fz = x[3 * i + 2] * w;
    if (s32) s32[i] = make_float4(float(fx), float(fy), float(fz), 0.f);
    if (s64) s64[i] = make_double4_32a(fx, fy, fz, 0.0);
}

// Chunk sums in fixed order, then (ct != 0) the coarse-target values of every used entry of the
// point's sphere interpolated to the point: u(nu_j) = sum_k w_k K_pe(nu_j . nu_k) u_k, the transposed
// coarse map (exact for fields of degree <= pe on the sphere), read coalesced as [coarse][fine].
template <typename Real>
__global__ void k_far_reduce(DevGeom g, const Real* __restrict__ partial, double pre, double* __restrict__ out,
                             int ct) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    const int sph = g.sid[i];
    const int pb = g.prob[sph];
    if (g.active && !g.active[pb]) return;
    const Problem pr = g.problems[pb];
    const long long mp = pr.p1 - pr.p0;
    const Real* base = partial + pr.poff + 3LL * (i - pr.p0);
    double sx = 0, sy = 0, sz = 0;
    if (!ct) {
        for (int c = 0; c < pr.nchunks; ++c) {
            const Real* q = base + 3LL * mp * c;
            sx += double(q[0]);
            sy += double(q[1]);
            sz += double(q[2]);
        }
    } else if (ct == 1) {
        // the grid entry's sums, then the listed coarse-target entries of the point's sphere by level
        const CoarseSet& cs = g.cs32;
        const float* o = cs.ctinterp + 3LL * ((long long)kCoarseLevels * g.M + i);
        sx = double(o[0]);
        sy = double(o[1]);
        sz = double(o[2]);
        for (int l = 0; l < kCoarseLevels; ++l) {
            if (!cs.ctused[sph * kCoarseLevels + l]) continue;
            o = cs.ctinterp + 3LL * ((long long)l * g.M + i);
            sx += double(o[0]);
            sy += double(o[1]);
            sz += double(o[2]);
        }
    } else {
        // the float-float set's slots: traction (ct 2) or single layer (ct 3) components
        const CoarseSet& cs = g.cshp;
        const int q = ct == 2 ? 0 : 3;
        const double* o = cs.ctinterpd + 6LL * ((long long)kCoarseLevels * g.M + i) + q;
        sx = o[0];
        sy = o[1];
        sz = o[2];
        for (int l = 0; l < kCoarseLevels; ++l) {
            if (!cs.ctused[sph * kCoarseLevels + l]) continue;
            o = cs.ctinterpd + 6LL * ((long long)l * g.M + i) + q;
            sx += o[0];
            sy += o[1];
            sz += o[2];
        }
    }
    out[3 * i] += pre * sx;
    out[3 * i + 1] += pre * sy;
    out[3 * i + 2] += pre * sz;
}

}  // namespace

int launch_far_pack(const DevGeom& g, const double* x, double c, float4* src32, double4_32a* src64, bool fp32,
                    cudaStream_t st) {
    k_far_pack<<<(g.M + 255) / 256, 256, 0, st>>>(g, x, c, fp32 ? src32 : nullptr, fp32 ? nullptr : src64);
    return 1;
}

template <int TPT>
void launch_far32(const DevGeom& g, const FarItem* items, int nitems, bool trac, const float4* src32, float* partial,
                  cudaStream_t st) {
    if (TPT == 1) {
        if (trac) k_far32<true, 1><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
        else k_far32<false, 1><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
    } else {
        constexpr int NPK = TPT / 2 > 0 ? TPT / 2 : 1;
        if (trac) k_far32x2<true, NPK><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
        else k_far32x2<false, NPK><<<nitems, kFarThreads, 0, st>>>(g, items, src32, partial);
    }
}

int launch_far_field(const DevGeom& g, const FarItem* items, int nitems, bool trac, bool fp32, const float4* src32,
                     const double4_32a* src64, void* partial, cudaStream_t st, int tpt) {
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

int launch_coarse_src_df(const DevGeom& g, const float4* src2, cudaStream_t st) {
    if (g.cshp.ncent <= 0 || g.cshp.ncdesc <= 0) return 0;
    k_coarse_src_df<<<g.cshp.ncdesc, 128 * kCgGroupsD, 0, st>>>(g, src2);
    return 1;
}

int launch_coarse_src(const DevGeom& g, const float4* src32, cudaStream_t st) {
    if (g.cs32.ncent <= 0 || g.cs32.ncdesc <= 0) return 0;
    k_coarse_src<<<g.cs32.ncdesc, 128 * kCgGroups, 0, st>>>(g, src32);
    return 1;
}

int launch_coarse_src_tc(const DevGeom& g, const float4* src32, cudaStream_t st) {
    if (g.cs32.ncent <= 0 || g.cs32.ncdesc_tc <= 0) return 0;
    k_coarse_src_tc<<<dim3(g.cs32.ncdesc_tc, kCoarseTcSplit), 128, kCsTcSmem, st>>>(g, src32);
    return 1;
}

template <int KB>
void launch_rep(const DevGeom& g, const FarItem* items, int nitems, int nrep, int rep_M, bool trac,
                const float4* src32, float* partial, cudaStream_t st) {
    const dim3 grid(nitems, (nrep + KB - 1) / KB);
    if (trac) k_far32_rep<true, KB><<<grid, kFarThreads, 0, st>>>(g, items, nrep, rep_M, src32, partial);
    else k_far32_rep<false, KB><<<grid, kFarThreads, 0, st>>>(g, items, nrep, rep_M, src32, partial);
}

int launch_far_field_rep(const DevGeom& g, const FarItem* items, int nitems, int nrep, int rep_M, bool trac,
                         const float4* src32, float* partial, cudaStream_t st) {
    if (nitems <= 0 || nrep <= 0) return 0;
    if (nrep <= 2) launch_rep<2>(g, items, nitems, nrep, rep_M, trac, src32, partial, st);
    else if (nrep <= 4) launch_rep<4>(g, items, nitems, nrep, rep_M, trac, src32, partial, st);
    else launch_rep<8>(g, items, nitems, nrep, rep_M, trac, src32, partial, st);
    return 1;
}

int launch_far_field_df_rep(const DevGeom& g, const FarItem* items, int nitems, int nrep, int rep_M,
                            const float4* src2, double* partial, double* partial_sl, cudaStream_t st) {
    if (nitems <= 0 || nrep <= 0) return 0;
    if (nrep <= 2) {
        k_far_df_rep<2><<<dim3(nitems, 1), kFarThreads, 0, st>>>(g, items, nrep, rep_M, src2, partial, partial_sl);
    } else {
        k_far_df_rep<4><<<dim3(nitems, (nrep + 3) / 4), kFarThreads, 0, st>>>(g, items, nrep, rep_M, src2, partial,
                                                                            partial_sl);
    }
    return 1;
}

int launch_far_pack_df(const DevGeom& g, const double* x, double c, float4* src2, cudaStream_t st) {
    k_far_pack_df<<<(g.M + 255) / 256, 256, 0, st>>>(g, x, c, src2);
    return 1;
}

int launch_far_field_df(const DevGeom& g, const FarItem* items, int nitems, int kind, const float4* src2,
                        double* partial, double* partial_sl, cudaStream_t st) {
    if (nitems <= 0) return 0;
    // items carry 2 * kFarThreadsDF targets each (two packed targets per thread)
    if (kind == 2) k_far_dfx2<2><<<nitems, kFarThreadsDF, 0, st>>>(g, items, src2, partial, partial_sl);
    else if (kind == 1) k_far_dfx2<1><<<nitems, kFarThreadsDF, 0, st>>>(g, items, src2, partial, nullptr);
    else k_far_dfx2<0><<<nitems, kFarThreadsDF, 0, st>>>(g, items, src2, partial, nullptr);
    return 1;
}

int launch_ct_classify(const DevGeom& g, const CoarseSet& cs, cudaStream_t st) {
    if (cs.nctent <= 0) return 0;
    k_ct_classify<<<cs.nctent, 128, 0, st>>>(g, cs);
    return 1;
}

int launch_far_df_ct(const DevGeom& g, const CtWork* works, int nworks, const float4* src2, double* partial,
                     cudaStream_t st) {
    if (g.cshp.nctent <= 0) return 0;
    int n = 0;
    if (nworks > 0) {
        k_far_df_ct<<<nworks, kFarThreadsDF, 0, st>>>(g, works, src2, partial);
        ++n;
    }
    const int nblk = ((g.pmax + 1) * (2 * g.pmax + 2) + 127) / 128;  // the largest entry: a grid entry
    k_ct_sum_df<<<dim3(g.cshp.nctent, nblk), 128, 0, st>>>(g, partial);
    ++n;
    if (g.cshp.nctitile > 0) {
        k_ct_interp_df<<<g.cshp.nctitile, 128, 0, st>>>(g);
        ++n;
    }
    return n;
}

int launch_far_reduce(const DevGeom& g, const void* partial, bool fp32, double pre, double* out, cudaStream_t st,
                      int ct) {
    const int blocks = (g.M + 255) / 256;
    if (fp32) k_far_reduce<float><<<blocks, 256, 0, st>>>(g, static_cast<const float*>(partial), pre, out, ct);
    else k_far_reduce<double><<<blocks, 256, 0, st>>>(g, static_cast<const double*>(partial), pre, out, ct);
    return 1;
}

int launch_far_ct(const DevGeom& g, const CtWork* works, int nworks, bool trac, const float4* src32, float* partial,
                  cudaStream_t st) {
    if (g.cs32.nctent <= 0) return 0;
    int n = 0;
    if (nworks > 0) {  // entries without candidates have no items: their sums are zeros
        if (trac) k_far32_ct<true><<<nworks, kFarThreads, 0, st>>>(g, works, src32, partial);
        else k_far32_ct<false><<<nworks, kFarThreads, 0, st>>>(g, works, src32, partial);
        ++n;
    }
    const int nblk = ((g.pmax + 1) * (2 * g.pmax + 2) + 127) / 128;  // the largest entry: a grid entry
    k_ct_sum<<<dim3(g.cs32.nctent, nblk), 128, 0, st>>>(g, partial);
    ++n;
    if (g.cs32.nctitile > 0) {  // grid entries only: nothing to interpolate
        if (g.coarse_tc && g.cs32.nctitile_tc > 0)
            k_ct_interp_tc<<<g.cs32.nctitile_tc, 128, kCsTcSmem, st>>>(g);
        else
            k_ct_interp<<<g.cs32.nctitile, 128, 0, st>>>(g);
        ++n;
    }
    return n;
}

}  // namespace smob
