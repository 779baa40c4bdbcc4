// df.h — float-float ("df64") arithmetic on the FP32 pipes, shared by the far-field and near-field
// kernels of the high-precision passes.
//
// Each value is an unevaluated sum hi + lo of two floats (about 48 significant bits). GB300 issues
// FP32 instructions 58x faster than FP64 ones, so these error-free transformations (Knuth's two-sum,
// FMA-based exact products; Dekker 1971, Hida, Li and Bailey's double-double library, written here
// in our own code) give FP64-class results well below the FP64 pipe's cost. The _rn intrinsics keep
// every rounding explicit: the compiler may not contract a product into a later addition, which
// would break the transformations.
#pragma once

#include <cuda_runtime.h>

namespace smob {

// 1/sqrt(x) by one MUFU instruction (PTX rsqrt.approx.ftz: no denormal fix-up, the arguments are
// squared distances); the Newton step of df_rsqrt makes it float-float accurate
__device__ __forceinline__ float mufu_rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Elementwise primitives on one float or on two packed lanes (float2 -> FP32x2 instructions), every
// rounding explicit; a lane of a packed operation rounds exactly like the scalar one, so the scalar
// and packed forms of each helper below agree bit for bit per lane.
__device__ __forceinline__ float v_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float v_neg(float a) { return -a; }
__device__ __forceinline__ float v_sub(float a, float b) { return __fadd_rn(a, -b); }
__device__ __forceinline__ float v_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float v_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float v_rsqrt(float a) { return mufu_rsqrt(a); }
__device__ __forceinline__ float v_c(float, float c) { return c; }
__device__ __forceinline__ float2 v_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 v_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 v_sub(float2 a, float2 b) { return __fadd2_rn(a, v_neg(b)); }
__device__ __forceinline__ float2 v_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 v_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 v_rsqrt(float2 a) { return make_float2(mufu_rsqrt(a.x), mufu_rsqrt(a.y)); }
__device__ __forceinline__ float2 v_c(float2, float c) { return make_float2(c, c); }

template <typename T>
struct dfv {
    T h, l;
};
using df2 = dfv<float2>;
using df1 = dfv<float>;

template <typename T>
__device__ __forceinline__ dfv<T> two_sum(T a, T b) {
    const T s = v_add(a, b);
    const T bb = v_sub(s, a);
    return {s, v_add(v_sub(a, v_sub(s, bb)), v_sub(b, bb))};
}
// Products, dot products, squares and the reciprocal square root return unnormalised pairs
// (|lo| up to a few ulp of hi instead of half an ulp): every result feeds further products or the
// two_sum accumulators, whose error bounds this leaves at ~2^-44 relative, far below the 1e-10 the
// refinement residuals need, and each skipped renormalisation saves three instructions.
template <typename T>
__device__ __forceinline__ dfv<T> df_mul_u(dfv<T> a, dfv<T> b) {
    const T p = v_mul(a.h, b.h);
    const T e = v_fma(a.h, b.h, v_neg(p));
    return {p, v_fma(a.h, b.l, v_fma(a.l, b.h, e))};
}
template <typename T>
__device__ __forceinline__ dfv<T> df_dot3(dfv<T> a, dfv<T> b, dfv<T> c, dfv<T> d, dfv<T> e, dfv<T> f) {
    const T p0 = v_mul(a.h, b.h), p1 = v_mul(c.h, d.h), p2 = v_mul(e.h, f.h);
    T lo = v_add(v_add(v_fma(a.h, b.h, v_neg(p0)), v_fma(c.h, d.h, v_neg(p1))), v_fma(e.h, f.h, v_neg(p2)));
    lo = v_fma(a.h, b.l, v_fma(a.l, b.h, lo));
    lo = v_fma(c.h, d.l, v_fma(c.l, d.h, lo));
    lo = v_fma(e.h, f.l, v_fma(e.l, f.h, lo));
    const dfv<T> s01 = two_sum(p0, p1);
    const dfv<T> s = two_sum(s01.h, p2);
    return {s.h, v_add(v_add(s.l, s01.l), lo)};
}
template <typename T>
__device__ __forceinline__ dfv<T> df_sqr3(dfv<T> a, dfv<T> b, dfv<T> c) {
    const T p0 = v_mul(a.h, a.h), p1 = v_mul(b.h, b.h), p2 = v_mul(c.h, c.h);
    T lo = v_add(v_add(v_fma(a.h, a.h, v_neg(p0)), v_fma(b.h, b.h, v_neg(p1))), v_fma(c.h, c.h, v_neg(p2)));
    lo = v_fma(v_add(a.h, a.h), a.l, lo);
    lo = v_fma(v_add(b.h, b.h), b.l, lo);
    lo = v_fma(v_add(c.h, c.h), c.l, lo);
    const dfv<T> s01 = two_sum(p0, p1);
    const dfv<T> s = two_sum(s01.h, p2);
    return {s.h, v_add(v_add(s.l, s01.l), lo)};
}
template <typename T>
__device__ __forceinline__ dfv<T> df_rsqrt(dfv<T> x) {
    const T y = v_rsqrt(x.h);
    const T yy = v_mul(y, y);
    const T yye = v_fma(y, y, v_neg(yy));
    // x*y^2 = 1 - e, evaluated to double-float accuracy; one Newton step squares the error
    const T p = v_mul(x.h, yy);
    const T pe = v_fma(x.h, yy, v_neg(p));
    const T e = v_sub(v_sub(v_sub(v_c(y, 1.0f), p), pe), v_fma(x.h, yye, v_mul(x.l, yy)));
    return {y, v_mul(v_mul(v_c(y, 0.5f), y), e)};
}
// accumulator: hi part by two_sum, lo parts summed and folded in at the end
template <typename T>
__device__ __forceinline__ void df_acc(T& ah, T& al, dfv<T> v) {
    const dfv<T> s = two_sum(ah, v.h);
    ah = s.h;
    al = v_add(al, v_add(s.l, v.l));
}


}  // namespace smob
