// ewpt_internal.cuh -- shared device/host definitions of libewpt.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ewpt.h"
#include "physics.cuh"

#define EWPT_NFIELD 20  // phi(4) W(9) Y(3) Gamma(3) Sigma(1)
#define EWPT_NMOM 16    // momenta of phi, W, Y

// Lattice geometry of one periodic box.
struct Grid {
    int nx, ny, nz;
    int64_t S;  // nx*ny*nz
};

// Stencil coefficients, pre-divided by (60 dx) and dx^2:
//   d/dx f   = a1 (f1 - f-1) + a2 (f2 - f-2) + a3 (f3 - f-3)
//   lap f    = l0 f0 + l1 sum(f+-1) + l2 sum(f+-2) + l3 sum(f+-3)
// (diff_scheme.jl:157-311: 45/60, -9/60, 1/60 and 3/2, -3/20, 1/90, -49/18).
template <typename T>
struct StencilCoef {
    T a1, a2, a3;
    T l0, l1, l2, l3;
};

struct Ptr36 {
    const void* p[36];
};
struct MPtr36 {
    void* p[36];
};

// Wrapped relative offsets of the 6 stencil neighbours along one axis:
// [+1, +2, +3, -1, -2, -3].
__device__ __forceinline__ void axis_offsets(int i, int n, int stride, int* o) {
    o[0] = (i + 1 < n ? 1 : 1 - n) * stride;
    o[1] = (i + 2 < n ? 2 : 2 - n) * stride;
    o[2] = (i + 3 < n ? 3 : 3 - n) * stride;
    o[3] = (i - 1 >= 0 ? -1 : n - 1) * stride;
    o[4] = (i - 2 >= 0 ? -2 : n - 2) * stride;
    o[5] = (i - 3 >= 0 ? -3 : n - 3) * stride;
}

template <typename T>
PhysCoef<T> make_phys(const ewpt_params& p, double Jex, double gam) {
    PhysCoef<T> c;
    c.gw = (T)p.gw;
    c.gy = (T)p.gy;
    c.hgw = (T)(0.5 * p.gw);
    c.hgy = (T)(0.5 * p.gy);
    c.gp2 = (T)p.gp2;
    c.omgp2 = (T)(1.0 - p.gp2);
    c.lam2 = (T)(2.0 * p.lambda);
    c.vev2 = (T)(p.vev * p.vev);
    c.bW = (T)p.beta_w;
    c.bY = (T)p.beta_y;
    c.bW2 = (T)(2.0 * p.beta_w);
    c.bY2 = (T)(2.0 * p.beta_y);
    c.hJex = (T)(0.5 * Jex);
    c.gam = (T)gam;
    return c;
}

template <typename T>
StencilCoef<T> make_stencil(double dx) {
    StencilCoef<T> s;
    const double i60 = 1.0 / (60.0 * dx), i2 = 1.0 / (dx * dx);
    s.a1 = (T)(45.0 * i60);
    s.a2 = (T)(-9.0 * i60);
    s.a3 = (T)(1.0 * i60);
    s.l0 = (T)(3.0 * (-49.0 / 18.0) * i2);
    s.l1 = (T)(1.5 * i2);
    s.l2 = (T)(-0.15 * i2);
    s.l3 = (T)((1.0 / 90.0) * i2);
    return s;
}

// Host-side launchers (stage.cu, diag.cu, spectrum.cu, init.cu).
struct Fp32State {
    float* hi;  // [36][S]
    float* lo;  // [36][S]
};
struct Fp32Work {
    float* kacc;  // [36][S] RK4-weighted sum of the stage rates
    float* xa;    // [36][S] stage inputs (ping-pong)
    float* xb;
};

cudaError_t launch_rates_fp64(const Grid& g, const Ptr36& in, const MPtr36& out, const ewpt_params& p,
                              double Jex, double gam, cudaStream_t st);
// Launch shape of the stage kernels: (bx, by) threads over x and y, one z
// plane per grid slice; reg selects the register-budget variant (stage.cu).
struct Tiling {
    int bx, by, reg;
    int pair;  // FP32 form: 1 = two x-adjacent sites per thread (stage_pair.cu), needs nx even
};
constexpr Tiling kDefaultTiling{32, 4, 0, 0};
int tiling_max_threads(int reg);

cudaError_t launch_step_fp64(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                             const ewpt_params& p, double Jex, double gam, cudaStream_t st);
cudaError_t launch_step_fp32(const Grid& g, const Tiling& t, Fp32State y, Fp32Work w, const ewpt_params& p,
                             double Jex, double gam, cudaStream_t st);
cudaError_t launch_step_fp32_pair(const Grid& g, const Tiling& t, Fp32State y, Fp32Work w, const ewpt_params& p,
                                  double Jex, double gam, cudaStream_t st);
cudaError_t launch_fp32_split(const Grid& g, const double* src, Fp32State dst, cudaStream_t st);
cudaError_t launch_fp32_join(const Grid& g, Fp32State src, double* dst, cudaStream_t st);
