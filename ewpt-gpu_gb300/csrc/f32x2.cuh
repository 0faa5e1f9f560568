// f32x2.cuh -- packed pair-of-float arithmetic for two lattice sites at once.
//
// sm_100-class GPUs issue FADD2/FMUL2/FFMA2: one instruction operates on a
// pair of floats.  The FP32-form stage kernel gives each thread two
// x-adjacent sites and runs the ordinary templated physics (physics.cuh) on
// this pair type, so every flux operation is one packed instruction for two
// sites.  A product is kept unevaluated (Prod) until it meets an addition, so
// `a * b + c` becomes a single FFMA2 as the scalar compiler would contract it.
#pragma once
#include <cuda_runtime.h>

struct f2;
struct Prod;

struct f2 {
    float2 v;
    __host__ __device__ __forceinline__ f2() {}
    __host__ __device__ __forceinline__ f2(float2 x) : v(x) {}
    __host__ __device__ __forceinline__ explicit f2(float s) : v(make_float2(s, s)) {}
    __host__ __device__ __forceinline__ explicit f2(double s) : v(make_float2((float)s, (float)s)) {}
    __host__ __device__ __forceinline__ explicit f2(int s) : v(make_float2((float)s, (float)s)) {}
    __device__ __forceinline__ f2(const Prod& p);
    __device__ __forceinline__ f2& operator+=(const f2& b);
    __device__ __forceinline__ f2& operator-=(const f2& b);
    __device__ __forceinline__ f2& operator+=(const Prod& b);
    __device__ __forceinline__ f2& operator-=(const Prod& b);
};

struct Prod {
    float2 a, b;
    __device__ __forceinline__ float2 eval() const { return __fmul2_rn(a, b); }
};

__device__ __forceinline__ float2 neg2(float2 x) { return make_float2(-x.x, -x.y); }

__device__ __forceinline__ f2::f2(const Prod& p) : v(p.eval()) {}

// products
__device__ __forceinline__ Prod operator*(const f2& a, const f2& b) { return Prod{a.v, b.v}; }
__device__ __forceinline__ Prod operator*(const Prod& a, const f2& b) { return Prod{a.eval(), b.v}; }
__device__ __forceinline__ Prod operator*(const f2& a, const Prod& b) { return Prod{a.v, b.eval()}; }
__device__ __forceinline__ Prod operator*(const Prod& a, const Prod& b) { return Prod{a.eval(), b.eval()}; }
__device__ __forceinline__ Prod operator-(const Prod& p) { return Prod{neg2(p.a), p.b}; }

// sums
__device__ __forceinline__ f2 operator+(const f2& a, const f2& b) { return __fadd2_rn(a.v, b.v); }
__device__ __forceinline__ f2 operator-(const f2& a, const f2& b) { return __fadd2_rn(a.v, neg2(b.v)); }
__device__ __forceinline__ f2 operator-(const f2& a) { return neg2(a.v); }
__device__ __forceinline__ f2 operator+(const f2& x, const Prod& p) { return __ffma2_rn(p.a, p.b, x.v); }
__device__ __forceinline__ f2 operator+(const Prod& p, const f2& x) { return __ffma2_rn(p.a, p.b, x.v); }
__device__ __forceinline__ f2 operator+(const Prod& p, const Prod& q) { return __ffma2_rn(q.a, q.b, p.eval()); }
__device__ __forceinline__ f2 operator-(const f2& x, const Prod& p) { return __ffma2_rn(neg2(p.a), p.b, x.v); }
__device__ __forceinline__ f2 operator-(const Prod& p, const f2& x) { return __ffma2_rn(p.a, p.b, neg2(x.v)); }
__device__ __forceinline__ f2 operator-(const Prod& p, const Prod& q) { return __ffma2_rn(neg2(q.a), q.b, p.eval()); }

// one division per site in the physics (1/|Phi|^2): two scalar divides
__device__ __forceinline__ f2 operator/(const f2& a, const f2& b) {
    return make_float2(a.v.x / b.v.x, a.v.y / b.v.y);
}
__device__ __forceinline__ f2 operator/(const f2& a, const Prod& b) { return a / f2(b); }

__device__ __forceinline__ f2& f2::operator+=(const f2& b) { return *this = *this + b; }
__device__ __forceinline__ f2& f2::operator-=(const f2& b) { return *this = *this - b; }
__device__ __forceinline__ f2& f2::operator+=(const Prod& b) { return *this = *this + b; }
__device__ __forceinline__ f2& f2::operator-=(const Prod& b) { return *this = *this - b; }

// Error-free transformations on packed pairs (Knuth's TwoSum; the product
// error by one fused multiply-add), for the compensated stencils of the
// FP32 form's compensated mode (accessors.cuh PairAcc::grad_lap_c).
// s + e == a + b exactly (s or e may be the object a or b refers to)
__device__ __forceinline__ void two_sum2(const f2& a, const f2& b, f2& s, f2& e) {
    const f2 x = a, y = b;
    const f2 r = x + y;
    const f2 bb = r - x;
    e = (x - (r - bb)) + (y - bb);
    s = r;
}
// p + e == a * b exactly (p or e may be the object a or b refers to)
__device__ __forceinline__ void two_prod2(const f2& a, const f2& b, f2& p, f2& e) {
    const f2 x = a, y = b;
    const f2 r = f2(x * y);
    e = x * y - r;
    p = r;
}
