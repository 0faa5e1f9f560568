// ewpt_internal.cuh -- shared device/host definitions of libewpt.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ewpt.h"
#include "physics.cuh"

#define EWPT_NFIELD 20  // phi(4) W(9) Y(3) Gamma(3) Sigma(1)
#define EWPT_NMOM 16    // momenta of phi, W, Y

// Lattice geometry of one periodic box, or of one z-slab of it: with zg > 0
// the arrays hold zg ghost planes below and above the nz interior planes
// (S = nx*ny*(nz + 2 zg) is then the array stride) and the FP64 stage
// kernels read z neighbours from the ghost planes instead of wrapping.
struct Grid {
    int nx, ny, nz;
    int64_t S;  // nx*ny*nz, or the padded array stride of a slab
    int zg = 0;
    // FP64 stage launches over a window of z planes: the launch's block z
    // index b covers plane k0 + b (0 for whole-lattice launches)
    int k0 = 0;
};

// Storage of one FP32-form [36][.] array set: element (i, j, k) of array a
// at a*P + o0 + i + px*(j + py*k).  Plain layout (ensemble members): px = nx,
// py = ny, P = S, o0 = 0.  Ghosted layout (single-lattice FP32 form): every
// array is a padded box of px x (ny+6) x (nz+6) cells, the sites at x offset
// 4 and y, z offsets 3, the row pitch px a multiple of 32 floats (128 bytes)
// with at least 4 spare cells on each x face; the boxes start `lead` = 28
// floats into the buffer so that every row's first site sits on a 128-byte
// boundary.  The ghost cells hold the periodic images of the sites within
// reach of the opposite face (x: 4 cells, y and z: 3); launch_ghost_fill
// refreshes them after every kernel that writes a stencil source (stage
// inputs, the state high part), so a stencil reads its neighbours with no
// wrap and a tile together with its 3-site halo is one dense box (one TMA
// copy).  A buffer holds 36*P + 32 floats.
struct Layout {
    int px, py, pz;
    int gx, gyz;  // ghost widths: (4, 3) ghosted, (0, 0) plain
    int64_t P, o0;
    int lead;     // floats before array 0's padded box
    __host__ __device__ __forceinline__ int64_t at(int i, int j, int k) const {
        return o0 + i + (int64_t)px * (j + (int64_t)py * k);
    }
};
inline Layout plain_layout(const Grid& g) { return Layout{g.nx, g.ny, g.nz, 0, 0, g.S, 0, 0}; }
inline Layout ghost_layout(const Grid& g) {
    const int px = (g.nx + 8 + 31) / 32 * 32, py = g.ny + 6, pz = g.nz + 6, lead = 28;
    return Layout{px, py, pz, 4, 3, (int64_t)px * py * pz, lead + 4 + (int64_t)px * (3 + (int64_t)py * 3), lead};
}

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

// Rows of y per L2 chunk of the FP32 stage kernels' block walk.  A z plane's stencil reads
// planes k-3..k+3 of all 36 arrays; walking the lattice plane by plane over
// whole 256^2 planes keeps ~110 MB of inputs live, too close to the 126 MB
// L2 next to the streaming outputs, and 30% of the stencil loads went back
// to DRAM (12.8 ms per step at 256^3).  Chunks of 8/16/24/32/64 rows
// measured 11.96/11.36/11.16/11.09/11.56 ms per step.
constexpr int kChunkRows = 32;

// Block b of a 1-D grid over nbx x nby blocks per plane and nz planes,
// walked x fastest, then the block rows of one y chunk of ycb block rows,
// then z, then the chunks: one chunk's 7-plane working set of all 36 arrays
// stays in L2 while the chunk sweeps z.
__device__ __forceinline__ void chunk_walk(int b, int nbx, int nby, int nz, int ycb, int& bx, int& by, int& k) {
    bx = b % nbx;
    b /= nbx;
    const int c = b / (ycb * nz), rem = b - c * ycb * nz;
    const int yc = min(ycb, nby - c * ycb);
    by = c * ycb + rem % yc;
    k = rem / yc;
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
    // p.gw != 0 (ewpt_validate_params)
    c.gg = (T)(p.gp2 * p.gw);
    c.ggy = (T)(p.gp2 * p.gy);
    c.lam2h = (T)(2.0 * p.lambda / (0.5 * p.gw));
    c.hJexh = (T)(0.5 * Jex / (0.5 * p.gw));
    c.gamh = (T)(gam / (0.5 * p.gw));
    c.ryw = (T)(p.gy / p.gw);
    c.igw = (T)(1.0 / p.gw);
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
// One stage (1..4) of that step (z-slabs exchange ghost planes between stages).
cudaError_t launch_stage_fp64(const Grid& g, const Tiling& t, int stage, double* y, double* yn, double* xa,
                              double* xb, const ewpt_params& p, double Jex, double gam, cudaStream_t st);
// The same stage over the z planes [k0, k1) only: those sites' outputs are
// what a whole-lattice launch writes for them, bit for bit, and no other
// site is written.  Reads the stage input on planes [k0 - 3, k1 + 3)
// (periodic).  Lets a host-to-host step start stage 1 on the planes already
// uploaded and download the planes stage 4 has finished.
cudaError_t launch_stage_fp64_planes(const Grid& g, const Tiling& t, int stage, int k0, int k1, double* y,
                                     double* yn, double* xa, double* xb, const ewpt_params& p, double Jex,
                                     double gam, cudaStream_t st);
// FP64 stage and rates with the alternative stencil orders (stage_orders.cu)
cudaError_t launch_step_fp64_order(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                                   const ewpt_params& p, double Jex, double gam, cudaStream_t st);
cudaError_t launch_rates_fp64_order(const Grid& g, const Ptr36& in, const MPtr36& out, const ewpt_params& p,
                                    double Jex, double gam, cudaStream_t st);
// DF64 form (stage_dd.cu): y, yn, xa, xb hold float pairs (hi, lo).
cudaError_t launch_step_dd(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                           double* cur, const ewpt_params& p, double Jex, double gam, cudaStream_t st);
cudaError_t launch_to_dd(int64_t n, double* v, cudaStream_t st);  // in place: double -> (hi, lo)
cudaError_t launch_from_dd(int64_t n, const double* src, double* dst, cudaStream_t st);
cudaError_t launch_step_fp32(const Grid& g, const Layout& L, const Tiling& t, Fp32State y, Fp32Work w,
                             const ewpt_params& p, double Jex, double gam, cudaStream_t st);
// comp: the compensated mode (gauge Laplacians and auxiliary gradients compensated, stage_pair.cu)
cudaError_t launch_step_fp32_pair(const Grid& g, const Layout& L, const Tiling& t, Fp32State y, Fp32Work w,
                                  const ewpt_params& p, double Jex, double gam, cudaStream_t st, bool comp = false);
// Copy the face sites of all 36 arrays of a ghosted buffer into their
// periodic images (stage.cu); the x faces only if xfaces.
cudaError_t launch_ghost_fill(const Grid& g, const Layout& L, float* buf, cudaStream_t st, bool xfaces);
// FP64 [36][S] <-> FP32 hi/lo in layout L (the ghost images of hi refreshed on split).
cudaError_t launch_fp32_split(const Grid& g, const Layout& L, const double* src, Fp32State dst, cudaStream_t st);
cudaError_t launch_fp32_join(const Grid& g, const Layout& L, Fp32State src, double* dst, cudaStream_t st);
