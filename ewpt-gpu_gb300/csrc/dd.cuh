// dd.cuh -- double-float ("dd") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi)/2, carrying a 48-bit
// significand on the FP32 pipes.
//
// GB300 executes 64 FP32 operations for every FP64 operation, so the FP64
// form of the stage kernel is bound by its FP64 pipe.  The DF64 form runs the
// same physics template on this type instead: every operation is a short
// sequence of FP32 operations built on the error-free transformations of
// Knuth (TwoSum), Dekker (FastTwoSum) and the FMA product error, as in
// Hida, Li and Bailey's double-double library (QD) with the "sloppy"
// addition.  Relative error per operation ~2^-47 (FP64: 2^-53); the exponent
// range is FP32's.  The expressions are written so that no multiplication
// can be contracted into an addition by the compiler (products are explicit
// fmaf / multiplications whose results are used as-is).
#pragma once
#include <cuda_runtime.h>

struct dd {
    float hi, lo;
    dd() = default;
    __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit dd(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit dd(float f) : hi(f), lo(0.f) {}
    __host__ __device__ explicit dd(int i) : dd((double)i) {}
    __host__ __device__ explicit dd(float2 v) : hi(v.x), lo(v.y) {}
    __host__ __device__ float2 f2() const { return make_float2(hi, lo); }
};

// |a| >= |b| (or a == 0): s + e == a + b exactly
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
    const float s = a + b;
    return dd(s, b - (s - a));
}

__device__ __forceinline__ dd operator+(const dd& a, const dd& b) {
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);  // TwoSum error of the high parts
    e += a.lo + b.lo;
    return dd_fast_two_sum(s, e);
}
__device__ __forceinline__ dd operator-(const dd& a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(const dd& a, const dd& b) { return a + (-b); }

__device__ __forceinline__ dd operator*(const dd& a, const dd& b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);  // exact error of the high product
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return dd_fast_two_sum(p, e);
}

// quotient with one correction step (~2^-46 relative)
__device__ __forceinline__ dd operator/(const dd& a, const dd& b) {
    const float q1 = a.hi / b.hi;
    const dd r = a - dd(q1) * b;
    return dd_fast_two_sum(q1, r.hi / b.hi);
}

__device__ __forceinline__ dd& operator+=(dd& a, const dd& b) { return a = a + b; }
__device__ __forceinline__ dd& operator-=(dd& a, const dd& b) { return a = a - b; }
