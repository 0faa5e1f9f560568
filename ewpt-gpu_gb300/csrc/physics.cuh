// physics.cuh -- per-site right-hand side of the temporal-gauge SU(2)xU(1)
// Higgs system, templated on the arithmetic type T (double for the FP64
// form, float for the FP32 stencil/flux form).
//
// Same equations as rk4_step! (gpu-kernels-rk4/main_rk4.jl:52-661):
//   covariant derivatives  cov_derivs_temporal.jl:23-130
//   field strengths        field_strengths.jl:34-311
//   kt_phi_a               main_rk4.jl:337-407
//   kt_W_a_i               main_rk4.jl:409-560
//   kt_Y_i                 main_rk4.jl:562-581
//   k_field = momentum     main_rk4.jl:585-600
//   k_Gamma_a, k_Sigma     main_rk4.jl:603-655
// evaluated in a register-frugal order: every rate is affine in the spatial
// derivatives, so each array's gradient and Laplacian are taken together and
// folded into the rate accumulators right away (Higgs block, then one colour
// of W at a time, then Y), and each rate is handed to the sink as soon as it
// is final.  The reference's index pattern of the beta_W bracket of kt_phi
// (dW_1_3_dt, dW_1_4_dt in all three colour rows, main_rk4.jl:350-352) and
// the per-component damping term gamma*phi_a*(phi_a*pi_a)/|Phi|^2 (:349, with
// its 0/0 at |Phi| = 0) are kept.
//
// For (a, b, c) a cyclic permutation of the colours, the SU(2) rate reads
//   kt W^a_i = lap W^a_i - g sum_j (d_j W^b_i W^c_j - d_j W^c_i W^b_j)
//              - g sum_j (W^b_j F^c_ij - W^c_j F^b_ij) + J^a_i - d_i Gamma^a
//              - g (W^b_i Gamma^c - W^c_i Gamma^b) + beta terms
// which is kt_W_1_2 .. kt_W_3_4 of main_rk4.jl:409-560 term by term.
//
// Accessor `Acc`:  v(a)  value of array a (0..35, order of ewpt.h) at the site
//   grad(a, gx, gy, gz)            6th-order first derivatives
//   grad_lap(a, gx, gy, gz, lap)   first derivatives and Laplacian
//   div3(a)                        dx(a) + dy(a+1) + dz(a+2)
// Sink `out(a, rate)` receives rate a = d y_a / dt exactly once.
//
// PART splits the work between three launches when there are no beta terms:
// 0 = everything; 1 = the Higgs rates (20-23), handing the Higgs currents of
// kt W and kt Y to the sink (out.keep_current(3 a + i, J^a_i), slots 0-8;
// out.keep_current(9 + i, J^Y_i), slots 9-11); 2 = the SU(2) rates (24-32);
// 3 = the field, auxiliary and U(1) rates (0-19, 33-35).  Parts 2 and 3
// take the currents back (out.load_current).  The values are those of
// PART 0.
#pragma once

// Qualifier of the per-site arithmetic (here and in accessors.cuh).  The
// library compiles it for the device only; the operation counter of the test
// suite (oracle/opcount.cu) defines it as __host__ __device__ to run the same
// templates on the host with an operator-counting scalar type.
#ifndef EWPT_ARITH
#define EWPT_ARITH __device__ __forceinline__
#endif

#include <type_traits>

// Accessors that declare kCompGauge = true give the gauge fields'
// Laplacians and the auxiliaries' gradients as compensated pairs
// (grad_lap_c, grad_c; accessors.cuh PairAcc) and site_rates subtracts them
// before rounding (comp_diff); every other accessor takes the plain path.
template <class A, class = void>
struct CompGauge : std::false_type {};
template <class A>
struct CompGauge<A, std::void_t<decltype(A::kCompGauge)>> : std::integral_constant<bool, A::kCompGauge> {};

template <typename T>
struct PhysCoef {
    T gw, gy, hgw, hgy;  // g, g', g/2, g'/2
    T gp2, omgp2;        // gp2, 1-gp2
    T lam2, vev2;        // 2*lambda, vev^2
    T bW, bY, bW2, bY2;  // beta_W, beta_Y, 2*beta_W, 2*beta_Y
    T hJex, gam;         // Jex/2, damping gamma
    // derived, for rates accumulated in units of the couplings
    T gg, ggy;           // gp2*g, gp2*g'
    T lam2h, hJexh, gamh;// 2*lambda, Jex/2 and gamma over g/2
    T ryw, igw;          // g'/g, 1/g
};

// Covariant derivatives D_i phi_a (cov_derivs_temporal.jl:23-130) along one
// axis with gauge components W1 = W_1_i, W2 = W_2_i, W3 = W_3_i and the
// hypercharge component in units of g: Yr = (g'/g) Y_i, so that
// D = d + (g/2) (W terms + Yr terms).
template <typename T>
EWPT_ARITH void cov_deriv_s(T d1, T d2, T d3, T d4, T p1, T p2, T p3, T p4, T W1, T W2, T W3, T Yr, T hgw, T& D1,
                            T& D2, T& D3, T& D4) {
    D1 = d1 + hgw * (W1 * p4 - W2 * p3 + W3 * p2 + Yr * p2);
    D2 = d2 - hgw * (W1 * p3 + W2 * p4 + W3 * p1 + Yr * p1);
    D3 = d3 + hgw * (W1 * p2 + W2 * p1 - W3 * p4 + Yr * p4);
    D4 = d4 - hgw * (W1 * p1 - W2 * p2 - W3 * p3 + Yr * p3);
}

// The same with Y_i and g'/2 apart (the diagnostics).
template <typename T>
EWPT_ARITH void cov_deriv(T d1, T d2, T d3, T d4, T p1, T p2, T p3, T p4, T W1, T W2, T W3, T Y,
                                          T hgw, T hgy, T& D1, T& D2, T& D3, T& D4) {
    D1 = d1 + hgw * (W1 * p4 - W2 * p3 + W3 * p2) + hgy * (Y * p2);
    D2 = d2 - hgw * (W1 * p3 + W2 * p4 + W3 * p1) - hgy * (Y * p1);
    D3 = d3 + hgw * (W1 * p2 + W2 * p1 - W3 * p4) + hgy * (Y * p4);
    D4 = d4 - hgw * (W1 * p1 - W2 * p2 - W3 * p3) - hgy * (Y * p3);
}

template <typename T, bool BETA, class Acc, class Sink, int PART = 0>
EWPT_ARITH void site_rates(const Acc& A, const PhysCoef<T>& c, Sink& out) {
    static_assert(PART == 0 || !BETA, "the beta terms couple every block: PART 0 only");
    constexpr bool kHiggs = PART == 0 || PART == 1, kSU2 = PART == 0 || PART == 2,
                   kRest = PART == 0 || PART == 3;
    // compensated gauge stencils: kt W^a_i = (lap W^a_i - d_i Gamma^a) + g Q^a_i and
    // kt Y_i = (lap Y_i - d_i Sigma) + g' jY_i with each bracket formed before rounding
    constexpr bool kComp = CompGauge<Acc>::value;
    const T gw = c.gw, gy = c.gy, hgw = c.hgw;
    const T p1 = A.v(0), p2 = A.v(1), p3 = A.v(2), p4 = A.v(3);
    T W[3][3];  // W[a][i] = W_{a+1}_{i+2}
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) W[a][i] = A.v(4 + 3 * a + i);
    const T Y2 = A.v(13), Y3 = A.v(14), Y4 = A.v(15);
    const T G[3] = {A.v(16), A.v(17), A.v(18)};
    const T S = A.v(19);
    const T pt1 = A.v(20), pt2 = A.v(21), pt3 = A.v(22), pt4 = A.v(23);

    // ---- k_field = momentum (main_rk4.jl:585-600)
    if constexpr (kRest) {
#pragma unroll
        for (int a = 0; a < 16; ++a) out(a, A.v(20 + a));
    }

    // ---- k_Gamma_a, k_Sigma (main_rk4.jl:603-655): (1 - gp2) d_i pi^a_i + gp2 g rho^a
    if constexpr (kRest) {
        T Wt[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) Wt[a][i] = A.v(24 + 3 * a + i);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            // Higgs charge, then the gauge charge -(W^b . Wt^c - W^c . Wt^b)
            T q;
            if (a == 0) q = p1 * pt4 - p4 * pt1 + p3 * pt2 - p2 * pt3;
            else if (a == 1) q = p3 * pt1 - p1 * pt3 + p4 * pt2 - p2 * pt4;
            else q = p1 * pt2 - p2 * pt1 + p4 * pt3 - p3 * pt4;
            q = q - W[b][0] * Wt[cc][0] + W[cc][0] * Wt[b][0] - W[b][1] * Wt[cc][1] + W[cc][1] * Wt[b][1] -
                W[b][2] * Wt[cc][2] + W[cc][2] * Wt[b][2];
            out(16 + a, c.omgp2 * A.div3(24 + 3 * a) + c.gg * q);
        }
        out(19, c.omgp2 * A.div3(33) + c.ggy * (p1 * pt2 - p2 * pt1 + p3 * pt4 - p4 * pt3));
    }

    // ---- Higgs block: gradients, covariant derivatives, kt_phi (main_rk4.jl:337-407)
    // Every rate below is one accumulator that each product term enters with
    // a single fused multiply-add: the gauge terms of kt_phi are summed in
    // units of g/2 and those of kt_W in units of g, the coupling applied once
    // at the end.  The Higgs currents jW, jY are kept in units of g and g'.
    T ktp1, ktp2, ktp3, ktp4;
    T jW[3][3], jY[3];
    T cx = T(0), cy = T(0), cz = T(0), pdot = T(0);
    if constexpr (!kHiggs) {
        if constexpr (kSU2) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i) jW[a][i] = out.load_current(3 * a + i);
        }
        if constexpr (kRest) {
#pragma unroll
            for (int i = 0; i < 3; ++i) jY[i] = out.load_current(9 + i);
        }
    } else {
        T d1[3], d2[3], d3[3], d4[3], l1, l2, l3, l4;
        A.grad_lap(0, d1[0], d1[1], d1[2], l1);
        A.grad_lap(1, d2[0], d2[1], d2[2], l2);
        A.grad_lap(2, d3[0], d3[1], d3[2], l3);
        A.grad_lap(3, d4[0], d4[1], d4[2], l4);
        const T Yr[3] = {c.ryw * Y2, c.ryw * Y3, c.ryw * Y4};  // (g'/g) Y_i
        T D1[3], D2[3], D3[3], D4[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
            cov_deriv_s(d1[i], d2[i], d3[i], d4[i], p1, p2, p3, p4, W[0][i], W[1][i], W[2][i], Yr[i], hgw, D1[i],
                        D2[i], D3[i], D4[i]);
        // Higgs currents of kt_W (main_rk4.jl:415,432,449,...) and kt_Y (:563), over g and g'
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            jW[0][i] = p1 * D4[i] - p2 * D3[i] + p3 * D2[i] - p4 * D1[i];
            jW[1][i] = -p1 * D3[i] - p2 * D4[i] + p3 * D1[i] + p4 * D2[i];
            jW[2][i] = p1 * D2[i] - p2 * D1[i] - p3 * D4[i] + p4 * D3[i];
            jY[i] = p1 * D2[i] - p2 * D1[i] + p3 * D4[i] - p4 * D3[i];
        }
        if constexpr (PART == 1) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i) out.keep_current(3 * a + i, jW[a][i]);
#pragma unroll
            for (int i = 0; i < 3; ++i) out.keep_current(9 + i, jY[i]);
        }
        if (BETA) {
            pdot = pt1 * p1 + pt2 * p2 + pt3 * p3 + pt4 * p4;
            cx = d1[0] * p1 + d2[0] * p2 + d3[0] * p3 + d4[0] * p4;
            cy = d1[1] * p1 + d2[1] * p2 + d3[1] * p3 + d4[1] * p4;
            cz = d1[2] * p1 + d2[2] * p2 + d3[2] * p3 + d4[2] * p4;
        }
        // The gauge terms of kt_phi pair each gradient with its covariant
        // derivative, (g/2) W.d phi + (g/2) W.D phi (main_rk4.jl:337-407), so
        // they are taken once on the sums e = d + D (d is not needed after).
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            d1[i] += D1[i];
            d2[i] += D2[i];
            d3[i] += D3[i];
            d4[i] += D4[i];
        }
        const T mag = p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4;
        // over g/2: the potential and external source 2 lambda (|Phi|^2 - v^2) + Jex/2,
        // the damping gamma / |Phi|^2 (its 0/0 at |Phi| = 0 kept), the charges (g Gamma^3 +- g' Sigma)/2
        const T potg = c.lam2h * (mag - c.vev2) + c.hJexh;
        const T damp = c.gamh / mag;
        const T q12 = G[2] + c.ryw * S, q34 = c.ryw * S - G[2];
        T a1 = W[0][0] * d4[0] + W[0][1] * d4[1] + W[0][2] * d4[2] - W[1][0] * d3[0] - W[1][1] * d3[1] -
               W[1][2] * d3[2] + W[2][0] * d2[0] + W[2][1] * d2[1] + W[2][2] * d2[2] + Yr[0] * d2[0] +
               Yr[1] * d2[1] + Yr[2] * d2[2] + q12 * p2 - G[1] * p3 + G[0] * p4 - potg * p1 - damp * p1 * (p1 * pt1);
        ktp1 = l1 + hgw * a1;
        T a2 = -W[0][0] * d3[0] - W[0][1] * d3[1] - W[0][2] * d3[2] - W[1][0] * d4[0] - W[1][1] * d4[1] -
               W[1][2] * d4[2] - W[2][0] * d1[0] - W[2][1] * d1[1] - W[2][2] * d1[2] - Yr[0] * d1[0] -
               Yr[1] * d1[1] - Yr[2] * d1[2] - q12 * p1 - G[0] * p3 - G[1] * p4 - potg * p2 - damp * p2 * (p2 * pt2);
        ktp2 = l2 + hgw * a2;
        T a3 = W[0][0] * d2[0] + W[0][1] * d2[1] + W[0][2] * d2[2] + W[1][0] * d1[0] + W[1][1] * d1[1] +
               W[1][2] * d1[2] - W[2][0] * d4[0] - W[2][1] * d4[1] - W[2][2] * d4[2] + Yr[0] * d4[0] +
               Yr[1] * d4[1] + Yr[2] * d4[2] + q34 * p4 + G[1] * p1 + G[0] * p2 - potg * p3 - damp * p3 * (p3 * pt3);
        ktp3 = l3 + hgw * a3;
        T a4 = -W[0][0] * d1[0] - W[0][1] * d1[1] - W[0][2] * d1[2] + W[1][0] * d2[0] + W[1][1] * d2[1] +
               W[1][2] * d2[2] + W[2][0] * d3[0] + W[2][1] * d3[1] + W[2][2] * d3[2] - Yr[0] * d3[0] -
               Yr[1] * d3[1] - Yr[2] * d3[2] - q34 * p3 - G[0] * p1 + G[1] * p2 - potg * p4 - damp * p4 * (p4 * pt4);
        ktp4 = l4 + hgw * a4;
    }

    // ---- SU(2) block, one colour at a time (field_strengths.jl:34-224)
    //   kt W^a_i = lap W^a_i - d_i Gamma^a + g Q^a_i, Q accumulated over g
    T ktW[3][3];
    T F[3][3];  // F[b][0] = F^b_xy (W_b_23), [1] = F^b_xz (W_b_24), [2] = F^b_yz (W_b_34)
    if constexpr (kSU2) {
    T Q[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, cc = (a + 2) % 3;
#pragma unroll
        for (int i = 0; i < 3; ++i) Q[a][i] = jW[a][i] - W[b][i] * G[cc] + W[cc][i] * G[b];
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        T dW[3][3];  // dW[i][j] = d_j W^b_i
        if constexpr (kComp) {
            T Gh[3], Gl[3];
            A.grad_c(16 + b, Gh, Gl);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                T lh, ll;
                A.grad_lap_c(4 + 3 * b + i, dW[i][0], dW[i][1], dW[i][2], lh, ll);
                Q[b][i] = Q[b][i] + A.comp_diff(lh, ll, Gh[i], Gl[i]) * c.igw;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                T lap;
                A.grad_lap(4 + 3 * b + i, dW[i][0], dW[i][1], dW[i][2], lap);
                Q[b][i] = Q[b][i] + lap * c.igw;
            }
        }
        const int b1 = (b + 1) % 3, b2 = (b + 2) % 3;
        F[b][0] = dW[1][0] - dW[0][1] + gw * (W[b1][0] * W[b2][1] - W[b1][1] * W[b2][0]);
        F[b][1] = dW[2][0] - dW[0][2] + gw * (W[b1][0] * W[b2][2] - W[b1][2] * W[b2][0]);
        F[b][2] = dW[2][1] - dW[1][2] + gw * (W[b1][1] * W[b2][2] - W[b1][2] * W[b2][1]);
        // d_j W^b_i enters Q^{b-1}_i with -W^{b+1}_j and Q^{b+1}_i with +W^{b-1}_j
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            Q[b2][i] = Q[b2][i] - dW[i][0] * W[b1][0] - dW[i][1] * W[b1][1] - dW[i][2] * W[b1][2];
            Q[b1][i] = Q[b1][i] + dW[i][0] * W[b2][0] + dW[i][1] * W[b2][1] + dW[i][2] * W[b2][2];
        }
    }
    // -sum_j (W^b_j F^c_ij - W^c_j F^b_ij) with F_ij antisymmetric
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, cc = (a + 2) % 3;
        // i = x: j = y (F_xy), z (F_xz)
        Q[a][0] = Q[a][0] - W[b][1] * F[cc][0] + W[cc][1] * F[b][0] - W[b][2] * F[cc][1] + W[cc][2] * F[b][1];
        // i = y: j = x (F_yx = -F_xy), z (F_yz)
        Q[a][1] = Q[a][1] - W[cc][0] * F[b][0] + W[b][0] * F[cc][0] - W[b][2] * F[cc][2] + W[cc][2] * F[b][2];
        // i = z: j = x (F_zx = -F_xz), y (F_zy = -F_yz)
        Q[a][2] = Q[a][2] - W[cc][0] * F[b][1] + W[b][0] * F[cc][1] - W[cc][1] * F[b][2] + W[b][1] * F[cc][2];
    }
    // the coupling and the auxiliary gradient
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if constexpr (kComp) {  // the gradient is in Q already
            ktW[a][0] = gw * Q[a][0];
            ktW[a][1] = gw * Q[a][1];
            ktW[a][2] = gw * Q[a][2];
        } else {
            T gx, gy_, gz;
            A.grad(16 + a, gx, gy_, gz);
            ktW[a][0] = gw * Q[a][0] - gx;
            ktW[a][1] = gw * Q[a][1] - gy_;
            ktW[a][2] = gw * Q[a][2] - gz;
        }
    }

    }  // SU(2) block

    // ---- U(1) block (field_strengths.jl:281-311, main_rk4.jl:562-581)
    T ktY[3], FY[3];
    if constexpr (kRest) {
        T dY[3][3], lap[3];
        if constexpr (kComp) {
            T Sh[3], Sl[3];
            A.grad_c(19, Sh, Sl);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                T lh, ll;
                A.grad_lap_c(13 + i, dY[i][0], dY[i][1], dY[i][2], lh, ll);
                lap[i] = A.comp_diff(lh, ll, Sh[i], Sl[i]);  // lap Y_i - d_i Sigma
            }
        } else {
#pragma unroll
            for (int i = 0; i < 3; ++i) A.grad_lap(13 + i, dY[i][0], dY[i][1], dY[i][2], lap[i]);
        }
        FY[0] = dY[1][0] - dY[0][1];
        FY[1] = dY[2][0] - dY[0][2];
        FY[2] = dY[2][1] - dY[1][2];
        if constexpr (kComp) {
            ktY[0] = lap[0] + gy * jY[0];
            ktY[1] = lap[1] + gy * jY[1];
            ktY[2] = lap[2] + gy * jY[2];
        } else {
            T gx, gy_, gz;
            A.grad(19, gx, gy_, gz);
            ktY[0] = lap[0] + gy * jY[0] - gx;
            ktY[1] = lap[1] + gy * jY[1] - gy_;
            ktY[2] = lap[2] + gy * jY[2] - gz;
        }
    }

    // ---- beta (CP-odd) terms
    if (BETA) {
        T Wt[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) Wt[a][i] = A.v(24 + 3 * a + i);
        const T Yt2 = A.v(33), Yt3 = A.v(34), Yt4 = A.v(35);
        // dual field strength: B_x = F_yz, B_y = -F_xz, B_z = F_xy
        const T bWt = (Wt[0][0] * F[0][2] + Wt[0][1] * (-F[0][1]) + Wt[0][2] * F[0][0] +
                       Wt[1][0] * F[1][2] + Wt[0][1] * (-F[1][1]) + Wt[0][2] * F[1][0] +
                       Wt[2][0] * F[2][2] + Wt[0][1] * (-F[2][1]) + Wt[0][2] * F[2][0]);
        const T bYt = (Yt2 * FY[2] + Yt3 * (-FY[1]) + Yt4 * FY[0]);
        const T bsum = c.bW * bWt + c.bY * bYt;
        ktp1 += bsum * p1;
        ktp2 += bsum * p2;
        ktp3 += bsum * p3;
        ktp4 += bsum * p4;
        const T bwp = c.bW2 * pdot, byp = c.bY2 * pdot;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            ktW[a][0] += -bwp * F[a][2] + c.bW2 * (cy * Wt[a][2] - cz * Wt[a][1]);
            ktW[a][1] += bwp * F[a][1] + c.bW2 * (cz * Wt[a][0] - cx * Wt[a][2]);
            ktW[a][2] += -bwp * F[a][0] + c.bW2 * (cx * Wt[a][1] - cy * Wt[a][0]);
        }
        ktY[0] += -byp * FY[2] + c.bY2 * (cy * Yt4 - cz * Yt3);
        ktY[1] += byp * FY[1] + c.bY2 * (cz * Yt2 - cx * Yt4);
        ktY[2] += -byp * FY[0] + c.bY2 * (cx * Yt3 - cy * Yt2);
    }
    if constexpr (kHiggs) {
        out(20, ktp1);
        out(21, ktp2);
        out(22, ktp3);
        out(23, ktp4);
    }
    if constexpr (kSU2) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) out(24 + 3 * a + i, ktW[a][i]);
    }
    if constexpr (kRest) {
        out(33, ktY[0]);
        out(34, ktY[1]);
        out(35, ktY[2]);
    }
}
