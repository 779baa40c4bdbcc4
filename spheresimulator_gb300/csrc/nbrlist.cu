// nbrlist.cu — the near-pair neighbour list built on the GPU.
//
// Replaces the distributed neighbour search of MPI/NearInteraction.txx:400-460 for one GPU. The
// pair rule is the reference's (criterion at :430-447, with Rad = 1.5 a per sphere from
// BIE/SphereSTKSHOperator.cpp:547): an ordered pair (t, s) of spheres of the same problem is near
// iff 0 < |c_s - c_t|^2 < (1.5 a_s + 1.5 a_t)^2, strict on both sides. The list is CSR by target,
// sources ascending (the reference sorts its pairs by target; InteractionManager groups them so).
// Every product and sum is an explicitly rounded IEEE operation (no contraction into FMAs), so the
// decision at the boundary is the same as a host evaluation of the same expression in FP64.
//   k_nbr_count : per target sphere, its near sources (one thread per target, sources of its problem)
//   k_nbr_scan  : one CTA: exclusive scans of the counts (CSR offsets) and of "is a near source"
//                 (near-source slots: the rule is symmetric, so s is a source iff it has near pairs)
//   k_nbr_fill  : per target, its sources and near-singular flags (gap < 0.1 min radius), and the
//                 slot of every sphere
#include "smob_internal.h"

namespace smob {

namespace {

// |c_s - c_t|^2 and (1.5 a_s + 1.5 a_t)^2, rounded operation by operation
__device__ __forceinline__ void pair_terms(const double* __restrict__ c, const double* __restrict__ r, int t, int s,
                                           double& r2, double& rn2) {
    r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        const double d = __dsub_rn(c[3 * s + k], c[3 * t + k]);
        r2 = __dadd_rn(r2, __dmul_rn(d, d));
    }
    const double rn = __dadd_rn(__dmul_rn(1.5, r[s]), __dmul_rn(1.5, r[t]));
    rn2 = __dmul_rn(rn, rn);
}

__global__ void k_nbr_count(const double* __restrict__ c, const double* __restrict__ r, const int* __restrict__ prob,
                            const Problem* __restrict__ problems, int N, int* __restrict__ count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    const Problem pr = problems[prob[t]];
    int n = 0;
    for (int s = pr.s0; s < pr.s1; ++s) {
        double r2, rn2;
        pair_terms(c, r, t, s, r2, rn2);
        if (r2 > 0.0 && r2 < rn2) ++n;
    }
    count[t] = n;
}

// One CTA of 1024 threads: start[0..N] = exclusive scan of count (start[N] = pairs), slot_of[s] = the
// exclusive scan of (count[s] > 0) or -1, totals[0] = pairs, totals[1] = slots.
__global__ void __launch_bounds__(1024) k_nbr_scan(const int* __restrict__ count, int N, int* __restrict__ start,
                                                   int* __restrict__ slot_of, int* __restrict__ totals) {
    __shared__ int wsum[2][32];
    __shared__ int carry[2];
    if (threadIdx.x == 0) carry[0] = carry[1] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < N; base += 1024) {
        const int i = base + threadIdx.x;
        const int v0 = i < N ? count[i] : 0;
        const int v1 = i < N && count[i] > 0 ? 1 : 0;
        int x0 = v0, x1 = v1;  // inclusive warp scans
        for (int o = 1; o < 32; o <<= 1) {
            const int y0 = __shfl_up_sync(0xffffffffu, x0, o), y1 = __shfl_up_sync(0xffffffffu, x1, o);
            if (lane >= o) x0 += y0, x1 += y1;
        }
        if (lane == 31) wsum[0][warp] = x0, wsum[1][warp] = x1;
        __syncthreads();
        if (warp == 0) {
            int a = wsum[0][lane], b = wsum[1][lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int ya = __shfl_up_sync(0xffffffffu, a, o), yb = __shfl_up_sync(0xffffffffu, b, o);
                if (lane >= o) a += ya, b += yb;
            }
            wsum[0][lane] = a;  // inclusive over warps
            wsum[1][lane] = b;
        }
        __syncthreads();
        const int off0 = carry[0] + (warp ? wsum[0][warp - 1] : 0);
        const int off1 = carry[1] + (warp ? wsum[1][warp - 1] : 0);
        if (i < N) {
            start[i] = off0 + x0 - v0;
            slot_of[i] = v1 ? off1 + x1 - v1 : -1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry[0] += wsum[0][31];
            carry[1] += wsum[1][31];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        start[N] = carry[0];
        totals[0] = carry[0];
        totals[1] = carry[1];
    }
}

__global__ void k_nbr_fill(const double* __restrict__ c, const double* __restrict__ r, const int* __restrict__ prob,
                           const Problem* __restrict__ problems, int N, const int* __restrict__ start,
                           const int* __restrict__ slot_of, int* __restrict__ src, unsigned char* __restrict__ precise,
                           int* __restrict__ slot_sphere) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    if (slot_of[t] >= 0) slot_sphere[slot_of[t]] = t;
    const Problem pr = problems[prob[t]];
    int k = start[t];
    for (int s = pr.s0; s < pr.s1; ++s) {
        double r2, rn2;
        pair_terms(c, r, t, s, r2, rn2);
        if (!(r2 > 0.0 && r2 < rn2)) continue;
        src[k] = s;
        // surface gap below a tenth of the smaller radius: near-singular (FP64 quadrature in FP32 passes)
        const double gap = __dsub_rn(__dsub_rn(__dsqrt_rn(r2), r[s]), r[t]);
        precise[k] = gap < __dmul_rn(0.1, fmin(r[s], r[t])) ? 1 : 0;
        ++k;
    }
}

// Spheres of one problem that overlap or touch (|c_s - c_t| <= a_s + a_t, s > t): the first such pair
// in (t, s) order, as t * N + s, by atomicMin into *first (initialised to all ones).
__global__ void k_overlap(const double* __restrict__ c, const double* __restrict__ r, const int* __restrict__ prob,
                          const Problem* __restrict__ problems, int N, unsigned long long* __restrict__ first) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    const Problem pr = problems[prob[t]];
    for (int s = t + 1; s < pr.s1; ++s) {
        double r2, rn2;
        pair_terms(c, r, t, s, r2, rn2);
        if (__dsqrt_rn(r2) <= __dadd_rn(r[s], r[t])) {
            atomicMin(first, (unsigned long long)t * (unsigned long long)N + (unsigned long long)s);
            return;
        }
    }
}

}  // namespace

int launch_overlap_check(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                         unsigned long long* first, cudaStream_t st) {
    if (N <= 0) return 0;
    k_overlap<<<(N + 127) / 128, 128, 0, st>>>(centers, radii, prob, problems, N, first);
    return 1;
}

int launch_nbr_count(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                     int* count, cudaStream_t st) {
    if (N <= 0) return 0;
    k_nbr_count<<<(N + 127) / 128, 128, 0, st>>>(centers, radii, prob, problems, N, count);
    return 1;
}

int launch_nbr_scan(const int* count, int N, int* start, int* slot_of, int* totals, cudaStream_t st) {
    k_nbr_scan<<<1, 1024, 0, st>>>(count, N, start, slot_of, totals);
    return 1;
}

int launch_nbr_fill(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                    const int* start, const int* slot_of, int* src, unsigned char* precise, int* slot_sphere,
                    cudaStream_t st) {
    if (N <= 0) return 0;
    k_nbr_fill<<<(N + 127) / 128, 128, 0, st>>>(centers, radii, prob, problems, N, start, slot_of, src, precise,
                                                 slot_sphere);
    return 1;
}

}  // namespace smob
