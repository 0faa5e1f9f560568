// accessors.cuh -- neighbour access for the stage kernels.
//
// An accessor serves site_rates (physics.cuh) the values, 6th-order
// gradients and Laplacians of the 36 stage-input arrays at its site, reading
// global memory through the read-only path with the periodic wrap folded
// into the neighbour offsets.  The source of the 36 array pointers is a
// policy: SrcPtr36 (one pointer per array, kernel parameter) for a single
// lattice, SrcBase (base + a*S) for members of a batched ensemble.
#pragma once
#include "ewpt_internal.cuh"
#include "f32x2.cuh"

template <typename TL>
struct SrcPtr36 {
    const Ptr36& P;
    EWPT_ARITH const TL* arr(int a) const { return reinterpret_cast<const TL*>(P.p[a]); }
};

template <typename TL>
struct SrcBase {
    const TL* base;
    int64_t S;
    __device__ __forceinline__ const TL* arr(int a) const { return base + a * S; }
};

// [36][S] block with 36 S < 2^31: 32-bit array offsets
template <typename TL>
struct SrcBase32 {
    const TL* base;
    int S;
    __device__ __forceinline__ const TL* arr(int a) const { return base + a * S; }
};

// One site per thread; TL = stored type, T = arithmetic type.
template <typename TL, typename T, class Src>
struct SiteAcc {
    Src src;
    int c;
    int ox[6], oy[6], oz[6];
    StencilCoef<T> s;

    EWPT_ARITH T ld(int a, int off) const {
#ifdef __CUDA_ARCH__
        return (T)__ldg(src.arr(a) + (c + off));
#else
        return (T)src.arr(a)[c + off];
#endif
    }
    EWPT_ARITH T v(int a) const { return ld(a, 0); }
    EWPT_ARITH T d1(int a, const int* o) const {
        return s.a1 * (ld(a, o[0]) - ld(a, o[3])) + s.a2 * (ld(a, o[1]) - ld(a, o[4])) +
               s.a3 * (ld(a, o[2]) - ld(a, o[5]));
    }
    EWPT_ARITH void grad(int a, T& gx, T& gy, T& gz) const {
        gx = d1(a, ox);
        gy = d1(a, oy);
        gz = d1(a, oz);
    }
    EWPT_ARITH void grad_lap(int a, T& gx, T& gy, T& gz, T& lap) const {
        T s1, s2, s3;
        {
            const T p1 = ld(a, ox[0]), p2 = ld(a, ox[1]), p3 = ld(a, ox[2]);
            const T m1 = ld(a, ox[3]), m2 = ld(a, ox[4]), m3 = ld(a, ox[5]);
            gx = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            s1 = p1 + m1;
            s2 = p2 + m2;
            s3 = p3 + m3;
        }
        {
            const T p1 = ld(a, oy[0]), p2 = ld(a, oy[1]), p3 = ld(a, oy[2]);
            const T m1 = ld(a, oy[3]), m2 = ld(a, oy[4]), m3 = ld(a, oy[5]);
            gy = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            s1 += p1 + m1;
            s2 += p2 + m2;
            s3 += p3 + m3;
        }
        {
            const T p1 = ld(a, oz[0]), p2 = ld(a, oz[1]), p3 = ld(a, oz[2]);
            const T m1 = ld(a, oz[3]), m2 = ld(a, oz[4]), m3 = ld(a, oz[5]);
            gz = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            s1 += p1 + m1;
            s2 += p2 + m2;
            s3 += p3 + m3;
        }
        lap = s.l0 * v(a) + s.l1 * s1 + s.l2 * s2 + s.l3 * s3;
    }
    // dx(a) + dy(a+1) + dz(a+2), the nine differences summed in one chain
    EWPT_ARITH T div3(int a) const {
        T r = s.a1 * (ld(a, ox[0]) - ld(a, ox[3]));
        r = r + s.a2 * (ld(a, ox[1]) - ld(a, ox[4])) + s.a3 * (ld(a, ox[2]) - ld(a, ox[5]));
        r = r + s.a1 * (ld(a + 1, oy[0]) - ld(a + 1, oy[3])) + s.a2 * (ld(a + 1, oy[1]) - ld(a + 1, oy[4])) +
            s.a3 * (ld(a + 1, oy[2]) - ld(a + 1, oy[5]));
        return r + s.a1 * (ld(a + 2, oz[0]) - ld(a + 2, oz[3])) + s.a2 * (ld(a + 2, oz[1]) - ld(a + 2, oz[4])) +
               s.a3 * (ld(a + 2, oz[2]) - ld(a + 2, oz[5]));
    }

    // site (i, j, k) of an nx x ny x nz box; with zg > 0 interior plane k of
    // a z-slab whose zg ghost planes on each side hold the neighbours' planes
    __device__ __forceinline__ void place(int i, int j, int k, int nx, int ny, int nz, int zg = 0) {
        axis_offsets(i, nx, 1, ox);
        axis_offsets(j, ny, nx, oy);
        if (zg == 0) {
            c = i + nx * (j + ny * k);
            axis_offsets(k, nz, nx * ny, oz);
        } else {
            c = i + nx * (j + ny * (k + zg));
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                oz[d] = (d + 1) * nx * ny;
                oz[d + 3] = -(d + 1) * nx * ny;
            }
        }
    }
    // site (i, j, k) of a ghosted layout: y and z neighbours are plain
    // strides (ghost cells), x neighbours wrap (the x ghost cells are kept
    // only for the TMA-staged kernel)
    __device__ __forceinline__ void place_ghost(int i, int j, int k, int nx, const Layout& L) {
        c = (int)L.at(i, j, k);
        const int sy = L.px, sz = L.px * L.py;
        axis_offsets(i, nx, 1, ox);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            oy[d] = (d + 1) * sy;
            oy[d + 3] = -(d + 1) * sy;
            oz[d] = (d + 1) * sz;
            oz[d + 3] = -(d + 1) * sz;
        }
    }
};

// Two x-adjacent sites (i0, i0+1), i0 even, packed float pairs.  The x
// stencil reads the aligned pairs at i0-4, i0-2, i0, i0+2, i0+4 and re-pairs
// them into the +-1, +-2, +-3 neighbours; y and z neighbours are aligned
// pairs of the same x columns.  Needs nx even.
//
// COMP = true (the FP32 form's compensated mode) adds grad_lap_c / grad_c:
// the Laplacian and the gradient as unevaluated sums hi + lo, accumulated
// with error-free transformations from the FP32 stage input and the
// coefficients split into float pairs (sl holds their low parts), so their
// error is ~2^-44 of the terms instead of ~2^-24.  The physics takes the
// gauge fields' Laplacians and the auxiliaries' gradients this way and
// subtracts them (comp_diff) before rounding to FP32: for the longitudinal
// gauge modes the two nearly cancel, and FP32 rounding of each would leak
// into the transverse (magnetic) modes.
template <class Src, bool COMP = false>
struct PairAcc {
    static constexpr bool kCompGauge = COMP;
    Src src;
    int c;      // linear index of site i0 (even)
    int ox[4];  // float offsets of the x pairs at i0-4, i0-2, i0+2, i0+4 (wrapped)
    int oy[6], oz[6];
    StencilCoef<f2> s;
    StencilCoef<f2> sl;  // low parts of the coefficients (COMP only)

    __device__ __forceinline__ float2 ld(int a, int off) const {
        return __ldg(reinterpret_cast<const float2*>(src.arr(a) + (c + off)));
    }
    __device__ __forceinline__ f2 v(int a) const { return f2(ld(a, 0)); }
    __device__ __forceinline__ void xpairs(int a, f2& p1, f2& p2, f2& p3, f2& m1, f2& m2, f2& m3) const {
        const float2 qm2 = ld(a, ox[0]), qm1 = ld(a, ox[1]), q0 = ld(a, 0), qp1 = ld(a, ox[2]), qp2 = ld(a, ox[3]);
        p1 = f2(make_float2(q0.y, qp1.x));
        p2 = f2(qp1);
        p3 = f2(make_float2(qp1.y, qp2.x));
        m1 = f2(make_float2(qm1.y, q0.x));
        m2 = f2(qm1);
        m3 = f2(make_float2(qm2.y, qm1.x));
    }
    __device__ __forceinline__ f2 dx(int a) const {
        f2 p1, p2, p3, m1, m2, m3;
        xpairs(a, p1, p2, p3, m1, m2, m3);
        return s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
    }
    __device__ __forceinline__ f2 d1(int a, const int* o) const {
        return s.a1 * (f2(ld(a, o[0])) - f2(ld(a, o[3]))) + s.a2 * (f2(ld(a, o[1])) - f2(ld(a, o[4]))) +
               s.a3 * (f2(ld(a, o[2])) - f2(ld(a, o[5])));
    }
    __device__ __forceinline__ void grad(int a, f2& gx, f2& gy, f2& gz) const {
        gx = dx(a);
        gy = d1(a, oy);
        gz = d1(a, oz);
    }
    __device__ __forceinline__ void grad_lap(int a, f2& gx, f2& gy, f2& gz, f2& lap) const {
        f2 s1, s2, s3;
        {
            f2 p1, p2, p3, m1, m2, m3;
            xpairs(a, p1, p2, p3, m1, m2, m3);
            gx = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            s1 = p1 + m1;
            s2 = p2 + m2;
            s3 = p3 + m3;
        }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            const int* o = ax == 0 ? oy : oz;
            const f2 p1 = f2(ld(a, o[0])), p2 = f2(ld(a, o[1])), p3 = f2(ld(a, o[2]));
            const f2 m1 = f2(ld(a, o[3])), m2 = f2(ld(a, o[4])), m3 = f2(ld(a, o[5]));
            const f2 g = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            if (ax == 0)
                gy = g;
            else
                gz = g;
            s1 += p1 + m1;
            s2 += p2 + m2;
            s3 += p3 + m3;
        }
        lap = s.l0 * v(a) + s.l1 * s1 + s.l2 * s2 + s.l3 * s3;
    }
    __device__ __forceinline__ f2 div3(int a) const { return dx(a) + d1(a + 1, oy) + d1(a + 2, oz); }

    // ---- compensated stencils (COMP)
    // (sh, sl) += v
    __device__ __forceinline__ static void acc2(f2& sh, f2& slo, const f2& v) {
        f2 e;
        two_sum2(sh, v, sh, e);
        slo = slo + e;
    }
    // (h, l) = coefficient (ch + cl) times (xh + xl), to ~2^-44
    __device__ __forceinline__ static void mul_c(const f2& ch, const f2& cl, const f2& xh, const f2& xl, f2& h, f2& l) {
        two_prod2(ch, xh, h, l);
        l = l + ch * xl + cl * xh;
    }
    // the plain gradient and the compensated Laplacian (lh + ll)
    __device__ __forceinline__ void grad_lap_c(int a, f2& gx, f2& gy, f2& gz, f2& lh, f2& ll) const {
        f2 Sh[3], Sl[3];  // sum over the axes of (f(+k) + f(-k)), k = 1, 2, 3
        {
            f2 p1, p2, p3, m1, m2, m3;
            xpairs(a, p1, p2, p3, m1, m2, m3);
            gx = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            two_sum2(p1, m1, Sh[0], Sl[0]);
            two_sum2(p2, m2, Sh[1], Sl[1]);
            two_sum2(p3, m3, Sh[2], Sl[2]);
        }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            const int* o = ax == 0 ? oy : oz;
            const f2 p1 = f2(ld(a, o[0])), p2 = f2(ld(a, o[1])), p3 = f2(ld(a, o[2]));
            const f2 m1 = f2(ld(a, o[3])), m2 = f2(ld(a, o[4])), m3 = f2(ld(a, o[5]));
            const f2 g = s.a1 * (p1 - m1) + s.a2 * (p2 - m2) + s.a3 * (p3 - m3);
            if (ax == 0)
                gy = g;
            else
                gz = g;
            acc2(Sh[0], Sl[0], p1);
            acc2(Sh[0], Sl[0], m1);
            acc2(Sh[1], Sl[1], p2);
            acc2(Sh[1], Sl[1], m2);
            acc2(Sh[2], Sl[2], p3);
            acc2(Sh[2], Sl[2], m3);
        }
        // l0 f0 + l1 S1 + l2 S2 + l3 S3
        const f2 f0 = v(a);
        two_prod2(s.l0, f0, lh, ll);
        ll = ll + sl.l0 * f0;
        const f2 ch[3] = {s.l1, s.l2, s.l3}, cl[3] = {sl.l1, sl.l2, sl.l3};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f2 th, tl, e;
            mul_c(ch[k], cl[k], Sh[k], Sl[k], th, tl);
            two_sum2(lh, th, lh, e);
            ll = ll + (tl + e);
        }
    }
    // the compensated derivative along one axis from its six neighbour pairs
    __device__ __forceinline__ void d1_c(const f2& p1, const f2& p2, const f2& p3, const f2& m1, const f2& m2,
                                         const f2& m3, f2& h, f2& l) const {
        const f2 ah[3] = {s.a1, s.a2, s.a3}, al[3] = {sl.a1, sl.a2, sl.a3};
        const f2 p[3] = {p1, p2, p3}, m[3] = {m1, m2, m3};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f2 dh, dl, th, tl;
            two_sum2(p[k], -m[k], dh, dl);
            mul_c(ah[k], al[k], dh, dl, th, tl);
            if (k == 0) {
                h = th;
                l = tl;
            } else {
                f2 e;
                two_sum2(h, th, h, e);
                l = l + (tl + e);
            }
        }
    }
    // compensated gradient: gh[i] + gl[i]
    __device__ __forceinline__ void grad_c(int a, f2* gh, f2* gl) const {
        {
            f2 p1, p2, p3, m1, m2, m3;
            xpairs(a, p1, p2, p3, m1, m2, m3);
            d1_c(p1, p2, p3, m1, m2, m3, gh[0], gl[0]);
        }
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            const int* o = ax == 0 ? oy : oz;
            d1_c(f2(ld(a, o[0])), f2(ld(a, o[1])), f2(ld(a, o[2])), f2(ld(a, o[3])), f2(ld(a, o[4])),
                 f2(ld(a, o[5])), gh[ax + 1], gl[ax + 1]);
        }
    }
    // (xh + xl) - (yh + yl), rounded once
    __device__ __forceinline__ static f2 comp_diff(const f2& xh, const f2& xl, const f2& yh, const f2& yl) {
        f2 d, e;
        two_sum2(xh, -yh, d, e);
        return d + (e + (xl - yl));
    }

    __device__ __forceinline__ void place(int i0, int j, int k, int nx, int ny, int nz) {
        c = i0 + nx * (j + ny * k);
        ox[0] = (i0 - 4 >= 0 ? -4 : nx - 4);
        ox[1] = (i0 - 2 >= 0 ? -2 : nx - 2);
        ox[2] = (i0 + 2 < nx ? 2 : 2 - nx);
        ox[3] = (i0 + 4 < nx ? 4 : 4 - nx);
        axis_offsets(j, ny, nx, oy);
        axis_offsets(k, nz, nx * ny, oz);
    }
    // pair (i0, i0+1) of a ghosted layout (y, z from ghost cells, x wrapped)
    __device__ __forceinline__ void place_ghost(int i0, int j, int k, int nx, const Layout& L) {
        c = (int)L.at(i0, j, k);
        const int sy = L.px, sz = L.px * L.py;
        ox[0] = (i0 - 4 >= 0 ? -4 : nx - 4);
        ox[1] = (i0 - 2 >= 0 ? -2 : nx - 2);
        ox[2] = (i0 + 2 < nx ? 2 : 2 - nx);
        ox[3] = (i0 + 4 < nx ? 4 : 4 - nx);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            oy[d] = (d + 1) * sy;
            oy[d + 3] = -(d + 1) * sy;
            oz[d] = (d + 1) * sz;
            oz[d + 3] = -(d + 1) * sz;
        }
    }
};

template <typename T>
__host__ __device__ inline StencilCoef<f2> pair_stencil(const StencilCoef<T>& s) {
    return StencilCoef<f2>{f2(s.a1), f2(s.a2), f2(s.a3), f2(s.l0), f2(s.l1), f2(s.l2), f2(s.l3)};
}
// the parts the FP32 coefficients miss: c - (float)c of the FP64 coefficients
inline StencilCoef<f2> pair_stencil_lo(const StencilCoef<double>& d) {
    auto lo = [](double x) { return f2((float)(x - (double)(float)x)); };
    return StencilCoef<f2>{lo(d.a1), lo(d.a2), lo(d.a3), lo(d.l0), lo(d.l1), lo(d.l2), lo(d.l3)};
}

// Compensated accumulation (hi, lo) += p (TwoSum, then renormalise).
template <typename T>
__device__ __forceinline__ void acc_hilo(T& hi, T& lo, T p) {
    const T s = hi + p;
    const T bp = s - hi;
    const T e = (hi - (s - bp)) + (p - bp);
    const T t = lo + e;
    hi = s + t;
    lo = t - (hi - s);
}
