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

struct KrylovLaunch {
    const VecChunk* chunks;
    int nchunks;
    const Problem* problems;
    int P;
    double* partial;  // nchunks * max_nvec
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
int launch_givens(const KrylovLaunch& L, int j, int m, KrylovState* ks, double* H, double* g, double* cs, double* sn,
                  const double* hnorm, unsigned char* active, int maxit, cudaStream_t st);
int launch_trisolve(const KrylovLaunch& L, int m, const unsigned char* in_cycle, const KrylovState* ks, const double* H,
                    const double* g, double* y, int* kc, cudaStream_t st);

}  // namespace smob
