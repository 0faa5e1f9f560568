// stencil_n.cuh -- central-difference stencils of any order 2R (R = 1, 3, 4, 5, 6).
//
// The reference keeps one module per order in diff_scheme.jl
// (differentiations: 6th, :1-365; differentiations_8th_order :370-626;
// _10th_order :627-932; _12th_order :933-1365; _2nd_order :1366-1438) and
// selects one with `using` (main_rk4.jl:33-35).  Here the order is the
// parameter ewpt_params.stencil_order and the radius R a template argument.
// The coefficients are the modules' integer weights over their common
// denominators, pre-divided by dx and dx^2:
//   d/dx f = sum_d a[d-1] (f(+d) - f(-d))
//   lap f  = l[0] f(0) + sum_d l[d] (sum over axes of f(+d) + f(-d))
// with l[0] three times the per-axis centre weight.
#pragma once
#include "ewpt_internal.cuh"

template <typename T, int R>
struct StencilN {
    T a[R];
    T l[R + 1];
};

// radius of a stencil order; 0 for orders the library does not offer
__host__ __device__ constexpr int stencil_radius(int order) {
    return order == 2 ? 1 : order == 6 ? 3 : order == 8 ? 4 : order == 10 ? 5 : order == 12 ? 6 : 0;
}

// Integer weights and denominators of the modules (first derivative: +1..+R;
// second derivative: centre, +1..+R; both symmetric).
template <int R>
struct StencilWeights;
template <>
struct StencilWeights<1> {  // diff_scheme.jl:1372-1414
    static constexpr double d1[1] = {1.}, d1den = 2.;
    static constexpr double d2[2] = {-2., 1.}, d2den = 1.;
};
template <>
struct StencilWeights<3> {  // diff_scheme.jl:157-311
    static constexpr double d1[3] = {45., -9., 1.}, d1den = 60.;
    static constexpr double d2[4] = {-490., 270., -27., 2.}, d2den = 180.;
};
template <>
struct StencilWeights<4> {  // diff_scheme.jl:376-620
    static constexpr double d1[4] = {672., -168., 32., -3.}, d1den = 840.;
    static constexpr double d2[5] = {-14350., 8064., -1008., 128., -9.}, d2den = 5040.;
};
template <>
struct StencilWeights<5> {  // diff_scheme.jl:633-926
    static constexpr double d1[5] = {2100., -600., 150., -25., 2.}, d1den = 2520.;
    static constexpr double d2[6] = {-73766., 42000., -6000., 1000., -125., 8.}, d2den = 25200.;
};
template <>
struct StencilWeights<6> {  // diff_scheme.jl:939-1359
    static constexpr double d1[6] = {23760., -7425., 2200., -495., 72., -5.}, d1den = 27720.;
    static constexpr double d2[7] = {-2480478., 1425600., -222750., 44000., -7425., 864., -50.}, d2den = 831600.;
};

template <typename T, int R>
StencilN<T, R> make_stencil_n(double dx) {
    using W = StencilWeights<R>;
    StencilN<T, R> s;
    for (int d = 0; d < R; ++d) s.a[d] = (T)(W::d1[d] / (W::d1den * dx));
    s.l[0] = (T)(3.0 * W::d2[0] / (W::d2den * dx * dx));
    for (int d = 1; d <= R; ++d) s.l[d] = (T)(W::d2[d] / (W::d2den * dx * dx));
    return s;
}

// Wrapped relative offsets of the 2R neighbours along one axis:
// o[0..R-1] = +1..+R, o[R..2R-1] = -1..-R.
template <int R>
__device__ __forceinline__ void axis_offsets_n(int i, int n, int stride, int* o) {
#pragma unroll
    for (int d = 1; d <= R; ++d) {
        int p = i + d, m = i - d;
        p -= p >= n ? n : 0;
        m += m < 0 ? n : 0;
        o[d - 1] = (p - i) * stride;
        o[R + d - 1] = (m - i) * stride;
    }
}

// One site per thread on a plain [36][S] layout; interface of physics.cuh.
template <typename TL, typename T, class Src, int R>
struct SiteAccN {
    Src src;
    int c;
    int ox[2 * R], oy[2 * R], oz[2 * R];
    StencilN<T, R> s;

    __device__ __forceinline__ T ld(int a, int off) const { return (T)__ldg(src.arr(a) + (c + off)); }
    __device__ __forceinline__ T v(int a) const { return ld(a, 0); }
    __device__ __forceinline__ T d1(int a, const int* o) const {
        T r = s.a[0] * (ld(a, o[0]) - ld(a, o[R]));
#pragma unroll
        for (int d = 1; d < R; ++d) r = r + s.a[d] * (ld(a, o[d]) - ld(a, o[R + d]));
        return r;
    }
    __device__ __forceinline__ void grad(int a, T& gx, T& gy, T& gz) const {
        gx = d1(a, ox);
        gy = d1(a, oy);
        gz = d1(a, oz);
    }
    __device__ __forceinline__ void grad_lap(int a, T& gx, T& gy, T& gz, T& lap) const {
        T sum[R];
        const int* os[3] = {ox, oy, oz};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int* o = os[ax];
            T g = T(0);
#pragma unroll
            for (int d = 0; d < R; ++d) {
                const T p = ld(a, o[d]), m = ld(a, o[R + d]);
                g = d == 0 ? s.a[0] * (p - m) : g + s.a[d] * (p - m);
                sum[d] = ax == 0 ? p + m : sum[d] + (p + m);
            }
            if (ax == 0)
                gx = g;
            else if (ax == 1)
                gy = g;
            else
                gz = g;
        }
        T l = s.l[0] * v(a);
#pragma unroll
        for (int d = 0; d < R; ++d) l = l + s.l[d + 1] * sum[d];
        lap = l;
    }
    __device__ __forceinline__ T div3(int a) const { return d1(a, ox) + d1(a + 1, oy) + d1(a + 2, oz); }

    __device__ __forceinline__ void place(int i, int j, int k, int nx, int ny, int nz) {
        c = i + nx * (j + ny * k);
        axis_offsets_n<R>(i, nx, 1, ox);
        axis_offsets_n<R>(j, ny, nx, oy);
        axis_offsets_n<R>(k, nz, nx * ny, oz);
    }
};
