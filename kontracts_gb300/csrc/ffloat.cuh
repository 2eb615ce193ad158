// ffloat.cuh — float-float ("double-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// a 48-bit significand. GB300's FP64 pipe issues at ~1/64 of the FP32 rate, so
// a chain of dependent FP64 operations (a Gauss solve, a long reduction) is far
// slower than the same chain in float-float, whose operations are short runs of
// FP32 additions and FMAs.
//
// Building blocks (error-free transformations):
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2 (s + e = a + b exactly)
//   quick_two_sum  Dekker 1971 (the same when |a| >= |b|)
//   two_prod       a * b = p + e exactly with one FMA
// Addition and division follow the accurate variants of Hida, Li and Bailey,
// "Algorithms for quad-double precision floating point arithmetic" (2001),
// carried over from double-double to float-float. Every operation uses the _rn
// intrinsics so that no compiler contraction or reassociation changes them.
#pragma once

namespace kx {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_make(float a) { return ff{a, 0.0f}; }

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

__device__ __forceinline__ ff quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return ff{p, __fmaf_rn(a, b, -p)};
}

// accurate addition (both pairs of components summed error-free)
__device__ __forceinline__ ff ff_add(ff x, ff y) {
    ff s = two_sum(x.hi, y.hi);
    const ff t = two_sum(x.lo, y.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }

// float-float + float
__device__ __forceinline__ ff ff_add_f(ff x, float b) {
    ff s = two_sum(x.hi, b);
    s.lo = __fadd_rn(s.lo, x.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_mul(ff x, ff y) {
    ff p = two_prod(x.hi, y.hi);
    p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
    p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ ff ff_mul_f(ff x, float b) {
    ff p = two_prod(x.hi, b);
    p.lo = __fmaf_rn(x.lo, b, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

// x / y: a quotient estimate from the leading floats, refined twice with the
// exact remainder (Hida-Li-Bailey accurate division).
__device__ __forceinline__ ff ff_div(ff x, ff y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    ff r = ff_sub(x, ff_mul_f(y, q1));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    r = ff_sub(r, ff_mul_f(y, q2));
    const float q3 = __fdiv_rn(r.hi, y.hi);
    const ff q = quick_two_sum(q1, q2);
    return ff_add_f(q, q3);
}

__device__ __forceinline__ ff ff_abs(ff x) { return x.hi < 0.0f ? ff_neg(x) : x; }

// x > y
__device__ __forceinline__ bool ff_gt(ff x, ff y) { return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo); }

__device__ __forceinline__ ff ff_shfl(ff x, int src) {
    return ff{__shfl_sync(0xffffffffu, x.hi, src), __shfl_sync(0xffffffffu, x.lo, src)};
}

}  // namespace kx
