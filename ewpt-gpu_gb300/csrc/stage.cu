// stage.cu -- fused RK4 stage kernels.
//
// One launch = one stage of classical RK4 (gpu-kernels-rk4/main_rk4.jl:
// 6146-6437): the stage kernel rk4_step! (main_rk4.jl:52-661) with the
// reference's broadcast combination fused into its epilogue, so the 144
// broadcast kernels and ~72 temporary N^3 arrays of a reference step become
// four launches and no temporaries.  The stage input X is written once per
// stage by the previous launch; the periodic halo is a wrap of the neighbour
// offsets inside the kernel (no ghost cells, no halo exchange).
//
// FP64 form (reference accumulation order, FMA contracted):
//   stage 1: k = f(y);   yn = y  + k dt/6;  X2 = y + k dt/2
//   stage 2: k = f(X2);  yn = yn + k dt/3;  X3 = y + k dt/2
//   stage 3: k = f(X3);  yn = yn + k dt/3;  X4 = y + k dt
//   stage 4: k = f(X4);  y  = yn + k dt/6
// FP32 form (FP32 stencils and fluxes, compensated float hi/lo state):
//   stage 1:     kacc = k1;           X2 = y_hi + k1 dt/2
//   stage 2, 3:  kacc += 2 k_s;       X3 = y_hi + k2 dt/2,  X4 = y_hi + k3 dt
//   stage 4:     (y_hi, y_lo) += dt/6 (kacc + k4), compensated, in place
// (X_1 is y_hi itself).  Bytes per site-update: FP64 4608, FP32 2736.
#include <algorithm>

#include "accessors.cuh"

namespace {

// Register-budget variants of the stage kernels (launch bounds, blocks of at
// most 128 threads): 0 = registers at the compiler's choice (up to 255);
// 1 = at most 128 registers (4 blocks per SM); 2 = at most 168 registers (3
// blocks per SM).  The block shape (bx, by) is a launch parameter.
template <int REG>
struct RegBudget;
template <>
struct RegBudget<0> { static constexpr int kThreads = 128, kMinBlocks = 1; };
template <>
struct RegBudget<1> { static constexpr int kThreads = 128, kMinBlocks = 4; };
template <>
struct RegBudget<2> { static constexpr int kThreads = 128, kMinBlocks = 3; };

template <typename TL, typename T>
using GlobalAcc = SiteAcc<TL, T, SrcPtr36<TL>>;

template <typename TL, typename T>
__device__ __forceinline__ bool make_acc(const Grid& g, const StencilCoef<T>& sc, GlobalAcc<TL, T>& A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z + g.k0;
    if (i >= g.nx || j >= g.ny) return false;
    A.place(i, j, k, g.nx, g.ny, g.nz, g.zg);
    A.s = sc;
    return true;
}

// ------------------------------------------------------------- rk4_step!
struct RatesSink {
    const MPtr36& R;
    int c;
    __device__ __forceinline__ void operator()(int a, double r) const { reinterpret_cast<double*>(R.p[a])[c] = r; }
};

template <bool BETA>
__global__ void __launch_bounds__(256) k_rates_fp64(Grid g, const __grid_constant__ Ptr36 X,
                                                       const __grid_constant__ MPtr36 R, PhysCoef<double> pc,
                                                       StencilCoef<double> sc) {
    GlobalAcc<double, double> A{{X}};
    if (!make_acc(g, sc, A)) return;
    RatesSink out{R, A.c};
    site_rates<double, BETA>(A, pc, out);
}

// ------------------------------------------------------------- FP64 stage
template <int STAGE>
struct Fp64Sink {
    const GlobalAcc<double, double>& A;
    const double* __restrict__ y;
    double* yn;
    double* __restrict__ xn;
    double* acc_out;
    int64_t S;
    double w, h;
    __device__ __forceinline__ void operator()(int a, double r) const {
        const int64_t q = a * S + A.c;
        if (STAGE == 1) {
            const double ya = A.v(a);  // X1 == y
            yn[q] = fma(r, w, ya);
            xn[q] = fma(r, h, ya);
        } else if (STAGE < 4) {
            // yn[q] is read and then written by this thread only: the
            // read-only path lets these loads issue ahead of earlier stores
            yn[q] = fma(r, w, __ldg(yn + q));
            xn[q] = fma(r, h, __ldg(y + q));
        } else {
            acc_out[q] = fma(r, w, __ldg(yn + q));
        }
    }
};

template <int STAGE, bool BETA, int REG>
__global__ void __launch_bounds__(RegBudget<REG>::kThreads, RegBudget<REG>::kMinBlocks) k_stage_fp64(Grid g, const __grid_constant__ Ptr36 X,
                                                       const double* __restrict__ y, double* yn,
                                                       double* __restrict__ xn, double* acc_out,
                                                       PhysCoef<double> pc, StencilCoef<double> sc, double w,
                                                       double h) {
    GlobalAcc<double, double> A{{X}};
    if (!make_acc(g, sc, A)) return;
    Fp64Sink<STAGE> out{A, y, yn, xn, acc_out, g.S, w, h};
    site_rates<double, BETA>(A, pc, out);
}

// ------------------------------------------------------------- FP32 stage
// All five FP32 buffers use the ghosted layout L.  After each stage the
// ghost images of what it wrote (the next stage input, or the state high
// part after stage 4) are refreshed by k_ghost_fill, so every stencil reads
// its neighbours with no wrap.
struct Fp32Bufs {
    float* yhi;  // [36][P] state, high part (also the stage-1 stencil input)
    float* ylo;  // [36][P] state, low part
    float* kacc; // [36][P] RK4-weighted rate sum: k1, then k1 + 2 k2, then k1 + 2 k2 + 2 k3
};

template <int STAGE>
struct Fp32Sink {
    const GlobalAcc<float, float>& A;
    const Layout& L;
    Fp32Bufs b;
    float* __restrict__ xn;
    float h, w6;
    __device__ __forceinline__ void operator()(int a, float r) const {
        const int64_t q = a * L.P + A.c;
        if (STAGE == 1) {
            b.kacc[q] = r;
            xn[q] = A.v(a) + h * r;  // X1 == y_hi
        } else if (STAGE < 4) {
            // kacc[q], yhi[q], ylo[q] are read and then written by this thread
            // only: the read-only path lets the loads issue ahead of stores
            b.kacc[q] = __ldg(b.kacc + q) + 2.f * r;
            xn[q] = __ldg(b.yhi + q) + h * r;
        } else {
            const float s = __ldg(b.kacc + q) + r;
            float hi = __ldg(b.yhi + q), lo = __ldg(b.ylo + q);
            acc_hilo(hi, lo, w6 * s);
            b.yhi[q] = hi;
            b.ylo[q] = lo;
        }
    }
};

template <int STAGE, bool BETA, int REG>
__global__ void __launch_bounds__(RegBudget<REG>::kThreads, RegBudget<REG>::kMinBlocks)
    k_stage_fp32(const __grid_constant__ Grid g, const __grid_constant__ Layout L, const __grid_constant__ Ptr36 X,
                 Fp32Bufs b, float* __restrict__ xn, PhysCoef<float> pc, StencilCoef<float> sc, float h, float w6,
                 int nbx, int nby, int ycb) {
    int bx, by, k;
    chunk_walk(blockIdx.x, nbx, nby, g.nz, ycb, bx, by, k);
    const int i = bx * blockDim.x + threadIdx.x;
    const int j = by * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    GlobalAcc<float, float> A{{X}};
    A.place_ghost(i, j, k, g.nx, L);
    A.s = sc;
    Fp32Sink<STAGE> out{A, L, b, xn, h, w6};
    site_rates<float, BETA>(A, pc, out);
}

// FP64 [36][S] -> (hi, lo) in layout L (ghost cells left to k_ghost_fill).
__global__ void k_split(Grid g, Layout L, const double* __restrict__ src, float* __restrict__ hi,
                        float* __restrict__ lo) {
    const int64_t n = 36 * g.S;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / g.S);
        const int64_t c = q - a * g.S;
        const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((int64_t)g.nx * g.ny));
        const double v = src[q];
        const float h = (float)v;
        const int64_t d = a * L.P + L.at(i, j, k);
        hi[d] = h;
        lo[d] = (float)(v - (double)h);
    }
}

__global__ void k_join(Grid g, Layout L, const float* __restrict__ hi, const float* __restrict__ lo,
                       double* __restrict__ dst) {
    const int64_t n = 36 * g.S;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q / g.S);
        const int64_t c = q - a * g.S;
        const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((int64_t)g.nx * g.ny));
        const int64_t d = a * L.P + L.at(i, j, k);
        dst[q] = (double)hi[d] + (double)lo[d];
    }
}

// Ghost images of a ghosted buffer, one warp per work item over a grid of a
// few blocks per SM: first the y- and z-face rows (a warp copies one row of
// nx sites into one of the 3 + 3 ghost rows of an x-y plane, or into a row
// of one of the 3 + 3 ghost planes), then, if asked, the x faces (a warp
// serves 4 rows, 8 cells each: the 4 ghost cells before the row and the 4
// after it).  The x faces cost most of the time (16-byte pieces of every
// row, 0.86 GB of DRAM reads per launch at 256^3 with them against ~0.12 GB
// without), so only the TMA-staged kernel, whose boxes read them, keeps
// them; the other FP32 kernels wrap x in their neighbour offsets.  Every
// cell copies the site it is the periodic image of; the box edges and
// corners are left alone (no axis-aligned stencil reaches them).
__global__ void __launch_bounds__(256) k_ghost_fill(Grid g, Layout L, float* __restrict__ buf, int xfaces) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int px = L.px, pxy = L.px * L.py;
    const int lane = threadIdx.x & 31;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int per_a = 6 * (ny + nz);
    for (int r = w0; r < 36 * per_a; r += nw) {
        const int a = r / per_a, e = r - a * per_a;
        float* arr = buf + a * L.P + L.o0;  // site (0, 0, 0)
        int doff, soff;
        if (e < 6 * nz) {
            const int yg = e % 6, k = e / 6;
            doff = (yg < 3 ? yg - 3 : ny + yg - 3) * px + k * pxy;
            soff = (yg < 3 ? ny + yg - 3 : yg - 3) * px + k * pxy;
        } else {
            const int zg = (e - 6 * nz) % 6, j = (e - 6 * nz) / 6;
            doff = j * px + (zg < 3 ? zg - 3 : nz + zg - 3) * pxy;
            soff = j * px + (zg < 3 ? nz + zg - 3 : zg - 3) * pxy;
        }
        for (int i = lane; i < nx; i += 32) arr[doff + i] = arr[soff + i];
    }
    if (!xfaces) return;
    const int rows = ny * nz, quads = (36 * rows + 3) / 4;
    const int xg = lane & 7;
    const int di = xg < 4 ? xg - 4 : nx + xg - 4, si = xg < 4 ? nx + xg - 4 : xg - 4;
    for (int q = w0; q < quads; q += nw) {
        const int rr = 4 * q + (lane >> 3);
        if (rr >= 36 * rows) continue;
        const int a = rr / rows, row = rr - a * rows;
        float* base = buf + a * L.P + L.o0 + (row % ny) * px + (row / ny) * pxy;
        base[di] = base[si];
    }
}

inline dim3 grid_of(const Grid& g, const Tiling& t) {
    return dim3((g.nx + t.bx - 1) / t.bx, (g.ny + t.by - 1) / t.by, g.nz);
}

Ptr36 pack(const void* base, int64_t S, size_t elem) {
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = static_cast<const char*>(base) + (size_t)a * S * elem;
    return P;
}

}  // namespace

int tiling_max_threads(int reg) { return reg >= 0 && reg <= 2 ? 128 : 0; }

cudaError_t launch_rates_fp64(const Grid& g, const Ptr36& in, const MPtr36& out, const ewpt_params& p,
                              double Jex, double gam, cudaStream_t st) {
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const StencilCoef<double> sc = make_stencil<double>(p.dx);
    const bool beta = p.beta_w != 0.0 || p.beta_y != 0.0;
    if (beta)
        k_rates_fp64<true><<<grid_of(g, kDefaultTiling), dim3(32, 4), 0, st>>>(g, in, out, pc, sc);
    else
        k_rates_fp64<false><<<grid_of(g, kDefaultTiling), dim3(32, 4), 0, st>>>(g, in, out, pc, sc);
    return cudaGetLastError();
}

template <bool BETA, int REG>
static void step_fp64(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                      const PhysCoef<double>& pc, const StencilCoef<double>& sc, double dt, cudaStream_t st) {
    const dim3 gr = grid_of(g, t), bl(t.bx, t.by);
    k_stage_fp64<1, BETA, REG><<<gr, bl, 0, st>>>(g, pack(y, g.S, 8), y, yn, xa, nullptr, pc, sc, dt / 6., dt / 2.);
    k_stage_fp64<2, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xa, g.S, 8), y, yn, xb, nullptr, pc, sc, dt / 3., dt / 2.);
    k_stage_fp64<3, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xb, g.S, 8), y, yn, xa, nullptr, pc, sc, dt / 3., dt);
    k_stage_fp64<4, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xa, g.S, 8), y, yn, nullptr, y, pc, sc, dt / 6., 0.0);
}

// planes g.k0 .. g.k0 + nzl - 1
template <bool BETA, int REG>
static void stage_fp64(const Grid& g, const Tiling& t, int stage, double* y, double* yn, double* xa, double* xb,
                       const PhysCoef<double>& pc, const StencilCoef<double>& sc, double dt, cudaStream_t st,
                       int nzl) {
    dim3 gr = grid_of(g, t);
    gr.z = nzl;
    const dim3 bl(t.bx, t.by);
    switch (stage) {
        case 1: k_stage_fp64<1, BETA, REG><<<gr, bl, 0, st>>>(g, pack(y, g.S, 8), y, yn, xa, nullptr, pc, sc, dt / 6., dt / 2.); break;
        case 2: k_stage_fp64<2, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xa, g.S, 8), y, yn, xb, nullptr, pc, sc, dt / 3., dt / 2.); break;
        case 3: k_stage_fp64<3, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xb, g.S, 8), y, yn, xa, nullptr, pc, sc, dt / 3., dt); break;
        default: k_stage_fp64<4, BETA, REG><<<gr, bl, 0, st>>>(g, pack(xa, g.S, 8), y, yn, nullptr, y, pc, sc, dt / 6., 0.0);
    }
}

template <bool BETA>
static void stage_fp64_r(const Grid& g, const Tiling& t, int stage, double* y, double* yn, double* xa, double* xb,
                         const PhysCoef<double>& pc, const StencilCoef<double>& sc, double dt, cudaStream_t st,
                         int nzl) {
    if (t.reg == 1)
        stage_fp64<BETA, 1>(g, t, stage, y, yn, xa, xb, pc, sc, dt, st, nzl);
    else if (t.reg == 2)
        stage_fp64<BETA, 2>(g, t, stage, y, yn, xa, xb, pc, sc, dt, st, nzl);
    else
        stage_fp64<BETA, 0>(g, t, stage, y, yn, xa, xb, pc, sc, dt, st, nzl);
}

cudaError_t launch_stage_fp64(const Grid& g, const Tiling& t, int stage, double* y, double* yn, double* xa,
                              double* xb, const ewpt_params& p, double Jex, double gam, cudaStream_t st) {
    Grid gw = g;
    gw.k0 = 0;
    return launch_stage_fp64_planes(gw, t, stage, 0, g.nz, y, yn, xa, xb, p, Jex, gam, st);
}

cudaError_t launch_stage_fp64_planes(const Grid& g, const Tiling& t, int stage, int k0, int k1, double* y,
                                     double* yn, double* xa, double* xb, const ewpt_params& p, double Jex,
                                     double gam, cudaStream_t st) {
    if (k0 < 0 || k1 > g.nz || k0 >= k1) return k0 == k1 ? cudaSuccess : cudaErrorInvalidValue;
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const StencilCoef<double> sc = make_stencil<double>(p.dx);
    Grid gw = g;
    gw.k0 = k0;
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        stage_fp64_r<true>(gw, t, stage, y, yn, xa, xb, pc, sc, p.dt, st, k1 - k0);
    else
        stage_fp64_r<false>(gw, t, stage, y, yn, xa, xb, pc, sc, p.dt, st, k1 - k0);
    return cudaGetLastError();
}

template <bool BETA>
static void step_fp64_r(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                        const PhysCoef<double>& pc, const StencilCoef<double>& sc, double dt, cudaStream_t st) {
    if (t.reg == 1)
        step_fp64<BETA, 1>(g, t, y, yn, xa, xb, pc, sc, dt, st);
    else if (t.reg == 2)
        step_fp64<BETA, 2>(g, t, y, yn, xa, xb, pc, sc, dt, st);
    else
        step_fp64<BETA, 0>(g, t, y, yn, xa, xb, pc, sc, dt, st);
}

cudaError_t launch_step_fp64(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                             const ewpt_params& p, double Jex, double gam, cudaStream_t st) {
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const StencilCoef<double> sc = make_stencil<double>(p.dx);
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        step_fp64_r<true>(g, t, y, yn, xa, xb, pc, sc, p.dt, st);
    else
        step_fp64_r<false>(g, t, y, yn, xa, xb, pc, sc, p.dt, st);
    return cudaGetLastError();
}

// FP32 form: stage inputs ping-pong between xa and xb.
template <bool BETA, int REG>
static void step_fp32(const Grid& g, const Layout& L, const Tiling& t, Fp32Bufs b, float* xa, float* xb,
                      const PhysCoef<float>& pc, const StencilCoef<float>& sc, double dt, cudaStream_t st) {
    const int nbx = (g.nx + t.bx - 1) / t.bx, nby = (g.ny + t.by - 1) / t.by;
    const int ycb = std::max(1, kChunkRows / t.by);
    const dim3 gr(nbx * nby * g.nz), bl(t.bx, t.by);
    const float h2 = (float)(dt / 2.), h1 = (float)dt, w6 = (float)(dt / 6.);
#define EWPT_WALK nbx, nby, ycb
    k_stage_fp32<1, BETA, REG><<<gr, bl, 0, st>>>(g, L, pack(b.yhi, L.P, 4), b, xa, pc, sc, h2, w6, EWPT_WALK);
    launch_ghost_fill(g, L, xa, st, false);
    k_stage_fp32<2, BETA, REG><<<gr, bl, 0, st>>>(g, L, pack(xa, L.P, 4), b, xb, pc, sc, h2, w6, EWPT_WALK);
    launch_ghost_fill(g, L, xb, st, false);
    k_stage_fp32<3, BETA, REG><<<gr, bl, 0, st>>>(g, L, pack(xb, L.P, 4), b, xa, pc, sc, h1, w6, EWPT_WALK);
    launch_ghost_fill(g, L, xa, st, false);
    k_stage_fp32<4, BETA, REG><<<gr, bl, 0, st>>>(g, L, pack(xa, L.P, 4), b, nullptr, pc, sc, 0.f, w6, EWPT_WALK);
    launch_ghost_fill(g, L, b.yhi, st, false);
#undef EWPT_WALK
}

template <bool BETA>
static void step_fp32_r(const Grid& g, const Layout& L, const Tiling& t, Fp32Bufs b, float* xa, float* xb,
                        const PhysCoef<float>& pc, const StencilCoef<float>& sc, double dt, cudaStream_t st) {
    if (t.reg == 1)
        step_fp32<BETA, 1>(g, L, t, b, xa, xb, pc, sc, dt, st);
    else if (t.reg == 2)
        step_fp32<BETA, 2>(g, L, t, b, xa, xb, pc, sc, dt, st);
    else
        step_fp32<BETA, 0>(g, L, t, b, xa, xb, pc, sc, dt, st);
}

cudaError_t launch_step_fp32(const Grid& g, const Layout& L, const Tiling& t, Fp32State y, Fp32Work w,
                             const ewpt_params& p, double Jex, double gam, cudaStream_t st) {
    if (L.gx == 0) return cudaErrorInvalidValue;  // the single-lattice kernels read ghost cells
    const PhysCoef<float> pc = make_phys<float>(p, Jex, gam);
    const StencilCoef<float> sc = make_stencil<float>(p.dx);
    Fp32Bufs b{y.hi, y.lo, w.kacc};
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        step_fp32_r<true>(g, L, t, b, w.xa, w.xb, pc, sc, p.dt, st);
    else
        step_fp32_r<false>(g, L, t, b, w.xa, w.xb, pc, sc, p.dt, st);
    return cudaGetLastError();
}

cudaError_t launch_ghost_fill(const Grid& g, const Layout& L, float* buf, cudaStream_t st, bool xfaces) {
    if (L.gx == 0) return cudaSuccess;
    k_ghost_fill<<<152 * 8, 256, 0, st>>>(g, L, buf, xfaces ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_fp32_split(const Grid& g, const Layout& L, const double* src, Fp32State dst, cudaStream_t st) {
    k_split<<<1216, 256, 0, st>>>(g, L, src, dst.hi, dst.lo);
    return launch_ghost_fill(g, L, dst.hi, st, true);
}

cudaError_t launch_fp32_join(const Grid& g, const Layout& L, Fp32State src, double* dst, cudaStream_t st) {
    k_join<<<1216, 256, 0, st>>>(g, L, src.hi, src.lo, dst);
    return cudaGetLastError();
}
