// diag.cu -- fused snapshot diagnostics and EM/Higgs field extraction.
//
// The reference runs 13 kernels per snapshot, each writing an N^3 scratch
// array that is copied to the host and summed there (main_rk4.jl:6451-6805,
// kernels compute_PE!..compute_Az! at :1334-3528, B_2 at :3718-4250).  Here
// one kernel computes every density of a site and reduces them in FP64
// (warp shuffle, then shared memory, then one partial row per block); a
// second single-block kernel folds the partial rows.  Nothing N^3-sized is
// written and nothing leaves the device but the 22 reduced values.
#include <cmath>

#include "ewpt_ctx.cuh"
#include "stencil_n.cuh"

namespace {

constexpr int DX_ = 32, DY_ = 4, DT = DX_ * DY_;

struct DiagCoef {
    double gw, gy, hgw, hgy, lambda, vev2, sw, cw, bcoef;  // bcoef = 4 sin(th)/(gw vev^2)
    double four_sw_gw;                                      // 4 sin(th)/gw (B_2)
    double a[6];                                            // first-derivative weights / dx (radius R)
};

// Neighbour access on an FP64 [36][S] buffer, stencil radius R.
template <int R>
struct DAcc {
    const double* __restrict__ y;
    int64_t S;
    int c;
    int ox[2 * R], oy[2 * R], oz[2 * R];
    double a[R];
    __device__ __forceinline__ double ld(int q, int off) const { return __ldg(y + q * S + c + off); }
    __device__ __forceinline__ double v(int q) const { return ld(q, 0); }
    __device__ __forceinline__ double d1(int q, const int* o) const {
        double r = a[0] * (ld(q, o[0]) - ld(q, o[R]));
#pragma unroll
        for (int d = 1; d < R; ++d) r = r + a[d] * (ld(q, o[d]) - ld(q, o[R + d]));
        return r;
    }
    __device__ __forceinline__ double dx(int a) const { return d1(a, ox); }
    __device__ __forceinline__ double dy(int a) const { return d1(a, oy); }
    __device__ __forceinline__ double dz(int a) const { return d1(a, oz); }
};

// All snapshot densities of one site.
struct SiteDiag {
    double pe, ke, ge, eew, mew, eey, mey;
    double bx, by, bz, b2x, b2y, b2z, ax, ay, az;
    double modphi;
    double gw1, gw2, gw3, gy_, cw1, cw2, cw3, cy;
};

template <class DA>
__device__ __forceinline__ void site_diag(const DA& A, const DiagCoef& k, SiteDiag& o) {
    const double p1 = A.v(0), p2 = A.v(1), p3 = A.v(2), p4 = A.v(3);
    const double W12 = A.v(4), W13 = A.v(5), W14 = A.v(6);
    const double W22 = A.v(7), W23 = A.v(8), W24 = A.v(9);
    const double W32 = A.v(10), W33 = A.v(11), W34 = A.v(12);
    const double Y2 = A.v(13), Y3 = A.v(14), Y4 = A.v(15);
    const double t1 = A.v(20), t2 = A.v(21), t3 = A.v(22), t4 = A.v(23);
    const double gw = k.gw, gy = k.gy;
    double D[3][4];
    {
        const double W1[3] = {W12, W13, W14}, W2[3] = {W22, W23, W24}, W3[3] = {W32, W33, W34}, Y[3] = {Y2, Y3, Y4};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double d1 = i == 0 ? A.dx(0) : (i == 1 ? A.dy(0) : A.dz(0));
            const double d2 = i == 0 ? A.dx(1) : (i == 1 ? A.dy(1) : A.dz(1));
            const double d3 = i == 0 ? A.dx(2) : (i == 1 ? A.dy(2) : A.dz(2));
            const double d4 = i == 0 ? A.dx(3) : (i == 1 ? A.dy(3) : A.dz(3));
            cov_deriv(d1, d2, d3, d4, p1, p2, p3, p4, W1[i], W2[i], W3[i], Y[i], k.hgw, k.hgy, D[i][0], D[i][1],
                      D[i][2], D[i][3]);
        }
    }
    const double mag = p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4;
    const double dev = mag - k.vev2;
    o.pe = k.lambda * (dev * dev);                                   // compute_PE!  :1340
    o.ke = t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4;                   // compute_KE!  :1659
    double ge = 0;                                                    // compute_GE!  :1498
#pragma unroll
    for (int a = 0; a < 4; ++a) ge += D[0][a] * D[0][a] + D[1][a] * D[1][a] + D[2][a] * D[2][a];
    o.ge = ge;
    double eew = 0;                                                   // compute_EEW! :1817
#pragma unroll
    for (int a = 24; a < 33; ++a) eew += A.v(a) * A.v(a);
    o.eew = 0.5 * eew;
    const double F1_23 = A.dx(5) - A.dy(4) + gw * (W22 * W33 - W23 * W32);
    const double F1_24 = A.dx(6) - A.dz(4) + gw * (W22 * W34 - W24 * W32);
    const double F1_34 = A.dy(6) - A.dz(5) + gw * (W23 * W34 - W24 * W33);
    const double F2_23 = A.dx(8) - A.dy(7) + gw * (W32 * W13 - W33 * W12);
    const double F2_24 = A.dx(9) - A.dz(7) + gw * (W32 * W14 - W34 * W12);
    const double F2_34 = A.dy(9) - A.dz(8) + gw * (W33 * W14 - W34 * W13);
    const double F3_23 = A.dx(11) - A.dy(10) + gw * (W12 * W23 - W13 * W22);
    const double F3_24 = A.dx(12) - A.dz(10) + gw * (W12 * W24 - W14 * W22);
    const double F3_34 = A.dy(12) - A.dz(11) + gw * (W13 * W24 - W14 * W23);
    o.mew = 0.5 * (F1_23 * F1_23 + F1_24 * F1_24 + F1_34 * F1_34 + F2_23 * F2_23 + F2_24 * F2_24 +
                   F2_34 * F2_34 + F3_23 * F3_23 + F3_24 * F3_24 + F3_34 * F3_34);   // compute_MEW! :1978
    const double Yt2 = A.v(33), Yt3 = A.v(34), Yt4 = A.v(35);
    o.eey = 0.5 * (Yt2 * Yt2 + Yt3 * Yt3 + Yt4 * Yt4);             // compute_EEY! :2139
    const double Y_23 = A.dx(14) - A.dy(13);
    const double Y_24 = A.dx(15) - A.dz(13);
    const double Y_34 = A.dy(15) - A.dz(14);
    o.mey = 0.5 * (Y_23 * Y_23 + Y_24 * Y_24 + Y_34 * Y_34);       // compute_MEY! :2298

    // EM fields: n^a = Phi^dag sigma^a Phi / |Phi|^2 (main_rk4.jl:2455-2467)
    double n1 = 0, n2 = 0, n3 = 0;
    if (mag != 0.0) {
        const double im = 1.0 / mag;
        n1 = -2. * (p1 * p3 + p2 * p4) * im;
        n2 = 2. * (p2 * p3 - p1 * p4) * im;
        n3 = (-(p1 * p1) - (p2 * p2) + (p3 * p3) + (p4 * p4)) * im;
    }
    const double hx = D[1][0] * D[2][1] - D[1][1] * D[2][0] + D[1][2] * D[2][3] - D[1][3] * D[2][2];
    const double hy = D[2][0] * D[0][1] - D[2][1] * D[0][0] + D[2][2] * D[0][3] - D[2][3] * D[0][2];
    const double hz = D[0][0] * D[1][1] - D[0][1] * D[1][0] + D[0][2] * D[1][3] - D[0][3] * D[1][2];
    const double sx = k.sw * (n1 * F1_34 + n2 * F2_34 + n3 * F3_34) + k.cw * Y_34;
    const double sy = k.sw * (n1 * (-F1_24) + n2 * (-F2_24) + n3 * (-F3_24)) + k.cw * (-Y_24);
    const double sz = k.sw * (n1 * F1_23 + n2 * F2_23 + n3 * F3_23) + k.cw * Y_23;
    o.bx = -(sx + k.bcoef * hx);                                    // compute_Bx!  :2469
    o.by = -(sy + k.bcoef * hy);                                    // compute_By!  :2643
    o.bz = -(sz + k.bcoef * hz);                                    // compute_Bz!  :2817
    if (mag == 0.0) {                                               // compute_B_2_*! :3883
        o.b2x = o.b2y = o.b2z = 0.0;
    } else {
        const double c2 = k.four_sw_gw / (mag * mag);
        o.b2x = -(sx + c2 * hx);
        o.b2y = -(sy + c2 * hy);
        o.b2z = -(sz + c2 * hz);
    }
    o.ax = k.sw * (n1 * W12 + n2 * W22 + n3 * W32) + k.cw * Y2;     // compute_Ax!  :3179
    o.ay = k.sw * (n1 * W13 + n2 * W23 + n3 * W33) + k.cw * Y3;
    o.az = k.sw * (n1 * W14 + n2 * W24 + n3 * W34) + k.cw * Y4;
    o.modphi = sqrt(mag);

    // Gauss constraint: div(E) minus the charge of k_Gamma/k_Sigma (main_rk4.jl:603-655)
    const double Wt12 = A.v(24), Wt13 = A.v(25), Wt14 = A.v(26);
    const double Wt22 = A.v(27), Wt23 = A.v(28), Wt24 = A.v(29);
    const double Wt32 = A.v(30), Wt33 = A.v(31), Wt34 = A.v(32);
    const double q1 = gw * (-(W22 * Wt32 - W32 * Wt22) - (W23 * Wt33 - W33 * Wt23) - (W24 * Wt34 - W34 * Wt24)) +
                      gw * (p1 * t4 - p4 * t1 + p3 * t2 - p2 * t3);
    const double q2 = gw * (-(W32 * Wt12 - W12 * Wt32) - (W33 * Wt13 - W13 * Wt33) - (W34 * Wt14 - W14 * Wt34)) +
                      gw * (p3 * t1 - p1 * t3 + p4 * t2 - p2 * t4);
    const double q3 = gw * (-(W12 * Wt22 - W22 * Wt12) - (W13 * Wt23 - W23 * Wt13) - (W14 * Wt24 - W24 * Wt14)) +
                      gw * (p1 * t2 - p2 * t1 + p4 * t3 - p3 * t4);
    const double qY = gy * (p1 * t2 - p2 * t1 + p3 * t4 - p4 * t3);
    o.gw1 = (A.dx(24) + A.dy(25) + A.dz(26)) - q1;
    o.gw2 = (A.dx(27) + A.dy(28) + A.dz(29)) - q2;
    o.gw3 = (A.dx(30) + A.dy(31) + A.dz(32)) - q3;
    o.gy_ = (A.dx(33) + A.dy(34) + A.dz(35)) - qY;
    o.cw1 = A.v(16) - (A.dx(4) + A.dy(5) + A.dz(6));
    o.cw2 = A.v(17) - (A.dx(7) + A.dy(8) + A.dz(9));
    o.cw3 = A.v(18) - (A.dx(10) + A.dy(11) + A.dz(12));
    o.cy = A.v(19) - (A.dx(13) + A.dy(14) + A.dz(15));
}

// Reduction slots
enum { R_PE = 0, R_KE, R_GE, R_EEW, R_MEW, R_EEY, R_MEY, R_BX, R_BY, R_BZ, R_B2X, R_B2Y, R_B2Z,
       R_MOD, R_HEL, R_GW, R_GY, R_CW, R_CY, NSUM, R_MIN = NSUM, R_MAXGW, R_MAXGY, NRED };

template <int R>
__device__ __forceinline__ void make_dacc(const Grid& g, const double* y, const DiagCoef& kc, int i, int j, int k,
                                          DAcc<R>& A) {
    A.y = y;
    A.S = g.S;
    A.c = i + g.nx * (j + g.ny * k);
    axis_offsets_n<R>(i, g.nx, 1, A.ox);
    axis_offsets_n<R>(j, g.ny, g.nx, A.oy);
    axis_offsets_n<R>(k, g.nz, g.nx * g.ny, A.oz);
#pragma unroll
    for (int d = 0; d < R; ++d) A.a[d] = kc.a[d];
}

template <int R>
__global__ void __launch_bounds__(DT) k_diag_partial(Grid g, const double* __restrict__ y, DiagCoef kc,
                                                     double* __restrict__ part) {
    double acc[NRED];
#pragma unroll
    for (int q = 0; q < NSUM; ++q) acc[q] = 0.0;
    acc[R_MIN] = INFINITY;
    acc[R_MAXGW] = 0.0;
    acc[R_MAXGY] = 0.0;
    const int i = blockIdx.x * DX_ + threadIdx.x;
    const int j = blockIdx.y * DY_ + threadIdx.y;
    if (i < g.nx && j < g.ny) {
        for (int k = blockIdx.z; k < g.nz; k += gridDim.z) {
            DAcc<R> A;
            make_dacc<R>(g, y, kc, i, j, k, A);
            SiteDiag o;
            site_diag(A, kc, o);
            acc[R_PE] += o.pe;
            acc[R_KE] += o.ke;
            acc[R_GE] += o.ge;
            acc[R_EEW] += o.eew;
            acc[R_MEW] += o.mew;
            acc[R_EEY] += o.eey;
            acc[R_MEY] += o.mey;
            acc[R_BX] += o.bx * o.bx;
            acc[R_BY] += o.by * o.by;
            acc[R_BZ] += o.bz * o.bz;
            acc[R_B2X] += o.b2x * o.b2x;
            acc[R_B2Y] += o.b2y * o.b2y;
            acc[R_B2Z] += o.b2z * o.b2z;
            acc[R_MOD] += o.modphi;
            acc[R_HEL] += o.b2x * o.ax + o.b2y * o.ay + o.b2z * o.az;
            acc[R_GW] += o.gw1 * o.gw1 + o.gw2 * o.gw2 + o.gw3 * o.gw3;
            acc[R_GY] += o.gy_ * o.gy_;
            acc[R_CW] += o.cw1 * o.cw1 + o.cw2 * o.cw2 + o.cw3 * o.cw3;
            acc[R_CY] += o.cy * o.cy;
            acc[R_MIN] = fmin(acc[R_MIN], o.modphi);
            acc[R_MAXGW] = fmax(acc[R_MAXGW], fmax(fabs(o.gw1), fmax(fabs(o.gw2), fabs(o.gw3))));
            acc[R_MAXGY] = fmax(acc[R_MAXGY], fabs(o.gy_));
        }
    }
    // warp shuffle reduction
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int q = 0; q < NSUM; ++q) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], off);
        acc[R_MIN] = fmin(acc[R_MIN], __shfl_down_sync(0xffffffffu, acc[R_MIN], off));
        acc[R_MAXGW] = fmax(acc[R_MAXGW], __shfl_down_sync(0xffffffffu, acc[R_MAXGW], off));
        acc[R_MAXGY] = fmax(acc[R_MAXGY], __shfl_down_sync(0xffffffffu, acc[R_MAXGY], off));
    }
    __shared__ double sh[DT / 32][NRED];
    const int lane = threadIdx.x & 31, warp = (threadIdx.y * DX_ + threadIdx.x) >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NRED; ++q) sh[warp][q] = acc[q];
    __syncthreads();
    const int t = threadIdx.y * DX_ + threadIdx.x;
    if (t < NRED) {
        double v = sh[0][t];
        for (int w = 1; w < DT / 32; ++w) {
            const double u = sh[w][t];
            v = t < NSUM ? v + u : (t == R_MIN ? fmin(v, u) : fmax(v, u));
        }
        const int64_t b = blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
        part[b * NRED + t] = v;
    }
}

__global__ void k_diag_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
    __shared__ double sh[256];
    for (int q = 0; q < NRED; ++q) {
        double v = q < NSUM ? 0.0 : (q == R_MIN ? INFINITY : 0.0);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const double u = part[(int64_t)b * NRED + q];
            v = q < NSUM ? v + u : (q == R_MIN ? fmin(v, u) : fmax(v, u));
        }
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                const double u = sh[threadIdx.x + s];
                double& w = sh[threadIdx.x];
                w = q < NSUM ? w + u : (q == R_MIN ? fmin(w, u) : fmax(w, u));
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = sh[0];
        __syncthreads();
    }
}

// Writes one real field per component: which = 0 -> B (compute_Bx/By/Bz!),
// 1 -> B_2 (compute_B_2_*!), 2 -> Higgs phi_1..4, 3 -> the seven energy
// densities (compute_PE! .. compute_MEY!).
template <int R>
__global__ void __launch_bounds__(DT) k_fields(Grid g, const double* __restrict__ y, DiagCoef kc, int which,
                                               double* __restrict__ f) {
    const int i = blockIdx.x * DX_ + threadIdx.x;
    const int j = blockIdx.y * DY_ + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    for (int k = blockIdx.z; k < g.nz; k += gridDim.z) {
        const int64_t c = i + (int64_t)g.nx * (j + (int64_t)g.ny * k);
        if (which == 2) {
#pragma unroll
            for (int a = 0; a < 4; ++a) f[a * g.S + c] = y[a * g.S + c];
            continue;
        }
        DAcc<R> A;
        make_dacc<R>(g, y, kc, i, j, k, A);
        SiteDiag o;
        site_diag(A, kc, o);
        if (which == 3) {
            const double d[7] = {o.pe, o.ke, o.ge, o.eew, o.mew, o.eey, o.mey};
#pragma unroll
            for (int q = 0; q < 7; ++q) f[q * g.S + c] = d[q];
            continue;
        }
        f[c] = which == 0 ? o.bx : o.b2x;
        f[g.S + c] = which == 0 ? o.by : o.b2y;
        f[2 * g.S + c] = which == 0 ? o.bz : o.b2z;
    }
}

DiagCoef diag_coef(const ewpt_params& p) {
    DiagCoef k;
    k.gw = p.gw;
    k.gy = p.gy;
    k.hgw = 0.5 * p.gw;
    k.hgy = 0.5 * p.gy;
    k.lambda = p.lambda;
    k.vev2 = p.vev * p.vev;
    k.sw = std::sin(p.theta_w);
    k.cw = std::cos(p.theta_w);
    k.bcoef = 4. * k.sw / (p.gw * (p.vev * p.vev));
    k.four_sw_gw = 4. * k.sw / p.gw;
    const int R = stencil_radius(p.stencil_order);
    for (int d = 0; d < 6; ++d) k.a[d] = 0.0;
    switch (R) {
        case 1: { const auto s = make_stencil_n<double, 1>(p.dx); for (int d = 0; d < 1; ++d) k.a[d] = s.a[d]; break; }
        case 4: { const auto s = make_stencil_n<double, 4>(p.dx); for (int d = 0; d < 4; ++d) k.a[d] = s.a[d]; break; }
        case 5: { const auto s = make_stencil_n<double, 5>(p.dx); for (int d = 0; d < 5; ++d) k.a[d] = s.a[d]; break; }
        case 6: { const auto s = make_stencil_n<double, 6>(p.dx); for (int d = 0; d < 6; ++d) k.a[d] = s.a[d]; break; }
        default: {  // the 6th-order coefficients of the stage kernels
            const StencilCoef<double> s = make_stencil<double>(p.dx);
            k.a[0] = s.a1;
            k.a[1] = s.a2;
            k.a[2] = s.a3;
        }
    }
    return k;
}

void launch_partial(int R, dim3 gr, const Grid& g, const double* y, const DiagCoef& kc, double* part,
                    cudaStream_t st) {
    const dim3 bl(DX_, DY_);
    switch (R) {
        case 1: k_diag_partial<1><<<gr, bl, 0, st>>>(g, y, kc, part); break;
        case 4: k_diag_partial<4><<<gr, bl, 0, st>>>(g, y, kc, part); break;
        case 5: k_diag_partial<5><<<gr, bl, 0, st>>>(g, y, kc, part); break;
        case 6: k_diag_partial<6><<<gr, bl, 0, st>>>(g, y, kc, part); break;
        default: k_diag_partial<3><<<gr, bl, 0, st>>>(g, y, kc, part);
    }
}

dim3 diag_grid(const Grid& g) {
    const int bx = (g.nx + DX_ - 1) / DX_, by = (g.ny + DY_ - 1) / DY_;
    // about 8 resident blocks on each of the SMs, z folded into a loop
    int bz = (152 * 8 + bx * by - 1) / (bx * by);
    if (bz > g.nz) bz = g.nz;
    if (bz < 1) bz = 1;
    return dim3(bx, by, bz);
}

}  // namespace

int ewpt_ensure_scratch64(ewpt_ctx* c) {
    if (c->scratch64) return EWPT_OK;
    return ewpt_cuda_check(c, cudaMalloc(&c->scratch64, (size_t)36 * c->g.S * 8), "scratch64");
}

int ewpt_state64(ewpt_ctx* c, const double** out) {
    if (c->slab)
        return ewpt_fail(c, EWPT_ERR_STATE, "a slab holds part of a lattice: gather the state (ewpt_slabs_get_state)");
    if (c->p.precision == EWPT_FP64) {
        *out = c->y;
        return EWPT_OK;
    }
    int rc = ewpt_ensure_scratch64(c);
    if (rc) return rc;
    if (c->p.precision == EWPT_DF64) {
        rc = ewpt_cuda_check(c, launch_from_dd(36 * c->g.S, c->y, c->scratch64, c->st), "join");
    } else {
        rc = ewpt_tma_check(c);
        if (rc) return rc;
        rc = ewpt_cuda_check(c, launch_fp32_join(c->g, c->lay, c->y32, c->scratch64, c->st), "join");
    }
    if (rc) return rc;
    *out = c->scratch64;
    return EWPT_OK;
}

// Reduced sums of one state -> the 20-column snapshot row.
static void finish_row(const ewpt_params& p, int64_t S, const double* r, double* out) {
    const double vol = p.dx * p.dx * p.dx;
    for (int q = 0; q < 7; ++q) out[q] = r[q] * vol;
    out[7] = (0.5 * (r[R_BX] + r[R_BY] + r[R_BZ])) * vol;
    out[8] = (0.5 * (r[R_B2X] + r[R_B2Y] + r[R_B2Z])) * vol;
    out[9] = r[R_MIN];
    out[10] = 0.0;
    out[11] = r[R_MOD] / (double)S;
    out[12] = r[R_HEL] * vol;
    out[13] = out[0] + out[1] + out[2] + out[3] + out[4] + out[5] + out[6];
    out[14] = std::sqrt(r[R_GW] * vol);
    out[15] = r[R_MAXGW];
    out[16] = std::sqrt(r[R_GY] * vol);
    out[17] = r[R_MAXGY];
    out[18] = std::sqrt(r[R_CW] * vol);
    out[19] = std::sqrt(r[R_CY] * vol);
}

// Launch the two reduction kernels for an FP64 [36][S] state; `part` holds
// grid-blocks * NRED doubles and `dres` NRED doubles, both device memory.
cudaError_t launch_diag(const Grid& g, const ewpt_params& p, const double* y, double* part, double* dres,
                        cudaStream_t st) {
    const dim3 gr = diag_grid(g);
    launch_partial(stencil_radius(p.stencil_order), gr, g, y, diag_coef(p), part, st);
    k_diag_final<<<1, 256, 0, st>>>(part, gr.x * gr.y * gr.z, dres);
    return cudaGetLastError();
}

int64_t diag_partial_count(const Grid& g) {
    const dim3 gr = diag_grid(g);
    return (int64_t)gr.x * gr.y * gr.z * NRED;
}

int diag_nred() { return NRED; }

// x-y tiles of the diagnostics grid: ceil(nx/32) * ceil(ny/4).
int64_t diag_tiles_xy(const Grid& g) { return (int64_t)((g.nx + DX_ - 1) / DX_) * ((g.ny + DY_ - 1) / DY_); }

// Same reduction as launch_diag on a grid of at most max_rows blocks (the z
// planes folded into each block's loop), for callers that supply a fixed
// scratch area of max_rows partial rows.  The caller checks
// diag_tiles_xy(g) <= max_rows.
cudaError_t launch_diag_bounded(const Grid& g, const ewpt_params& p, const double* y, double* part,
                                int64_t max_rows, double* dres, cudaStream_t st) {
    dim3 gr = diag_grid(g);
    const int64_t xy = (int64_t)gr.x * gr.y;
    int64_t bz = max_rows / xy;
    if (bz > (int64_t)gr.z) bz = gr.z;
    if (bz < 1) bz = 1;
    gr.z = (unsigned)bz;
    launch_partial(stencil_radius(p.stencil_order), gr, g, y, diag_coef(p), part, st);
    k_diag_final<<<1, 256, 0, st>>>(part, gr.x * gr.y * gr.z, dres);
    return cudaGetLastError();
}

void diag_finish_row(const ewpt_params& p, int64_t S, const double* r, double* out) { finish_row(p, S, r, out); }

cudaError_t launch_fields(const Grid& g, const ewpt_params& p, const double* y, int which, double* f,
                          cudaStream_t st) {
    const dim3 gr = diag_grid(g), bl(DX_, DY_);
    const DiagCoef kc = diag_coef(p);
    switch (stencil_radius(p.stencil_order)) {
        case 1: k_fields<1><<<gr, bl, 0, st>>>(g, y, kc, which, f); break;
        case 4: k_fields<4><<<gr, bl, 0, st>>>(g, y, kc, which, f); break;
        case 5: k_fields<5><<<gr, bl, 0, st>>>(g, y, kc, which, f); break;
        case 6: k_fields<6><<<gr, bl, 0, st>>>(g, y, kc, which, f); break;
        default: k_fields<3><<<gr, bl, 0, st>>>(g, y, kc, which, f);
    }
    return cudaGetLastError();
}

extern "C" int32_t ewpt_field_components(int32_t field) {
    switch (field) {
        case EWPT_FIELD_B:
        case EWPT_FIELD_B2: return 3;
        case EWPT_FIELD_HIGGS: return 4;
        case EWPT_FIELD_DENSITY: return 7;
        default: return -1;
    }
}

extern "C" int ewpt_fields(ewpt_ctx* c, int32_t field, double* out, int32_t on_device) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    const int ncomp = ewpt_field_components(field);
    if (ncomp < 0) return ewpt_fail(c, EWPT_ERR_ARG, "field %d unknown", field);
    if (!out) return ewpt_fail(c, EWPT_ERR_ARG, "out is NULL");
    cudaSetDevice(c->p.device);
    const double* y;
    int rc = ewpt_state64(c, &y);
    if (rc) return rc;
    const size_t bytes = (size_t)ncomp * c->g.S * 8;
    double* f = out;
    cudaError_t e = cudaSuccess;
    if (!on_device) e = cudaMallocAsync(&f, bytes, c->st);
    const int which = field == EWPT_FIELD_B ? 0 : field == EWPT_FIELD_B2 ? 1 : field == EWPT_FIELD_HIGGS ? 2 : 3;
    if (e == cudaSuccess) e = launch_fields(c->g, c->p, y, which, f, c->st);
    if (!on_device && f != out) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, f, bytes, cudaMemcpyDeviceToHost, c->st);
        const cudaError_t ef = cudaFreeAsync(f, c->st);
        if (e == cudaSuccess) e = ef;
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    }
    return ewpt_cuda_check(c, e, "fields");
}

extern "C" int ewpt_diagnostics(ewpt_ctx* c, double out[EWPT_NDIAG]) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!out) return ewpt_fail(c, EWPT_ERR_ARG, "out is NULL");
    cudaSetDevice(c->p.device);
    const double* y;
    int rc = ewpt_state64(c, &y);
    if (rc) return rc;
    if (!c->red) {
        c->red_blocks = (int)(diag_partial_count(c->g) / NRED);
        rc = ewpt_cuda_check(c, cudaMalloc(&c->red, (size_t)diag_partial_count(c->g) * 8), "diag scratch");
        if (rc) return rc;
        rc = ewpt_cuda_check(c, cudaMalloc(&c->dres, 64 * 8), "diag result");
        if (rc) return rc;
    }
    cudaError_t e = launch_diag(c->g, c->p, y, c->red, c->dres, c->st);
    double r[NRED];
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, c->dres, sizeof r, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(c, e, "diagnostics");
    if (rc) return rc;
    finish_row(c->p, c->g.S, r, out);
    for (int q = 0; q < EWPT_NDIAG; ++q)
        if (!std::isfinite(out[q])) return ewpt_fail(c, EWPT_ERR_NONFINITE, "non-finite diagnostic column %d", q);
    return EWPT_OK;
}
