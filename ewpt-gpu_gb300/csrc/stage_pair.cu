// stage_pair.cu -- FP32-form RK4 stage kernels with two sites per thread.
//
// Same stage structure and arithmetic as k_stage_fp32 (stage.cu), but each
// thread owns the x-adjacent sites (i0, i0+1), i0 even, and runs the physics
// on packed float pairs (f32x2.cuh): every flux operation is one FFMA2 /
// FADD2 / FMUL2 for both sites, and every neighbour access is a float2 load.
// For the x stencil the pairs at i0-4, i0-2, i0, i0+2, i0+4 (five aligned
// float2 loads) are re-paired into the +-1, +-2, +-3 neighbour pairs; y and z
// neighbours are aligned float2 loads of the same x pair.  The buffers use
// the ghosted layout (ewpt_internal.cuh), so neighbours past a face are read
// from the ghost cells along y and z (refreshed by k_ghost_fill after each
// stage) and wrapped in the offsets along x.  Needs nx even.
#include <algorithm>

#include "accessors.cuh"

namespace {

template <int REG>
struct PairBudget;
template <>
struct PairBudget<0> { static constexpr int kThreads = 128, kMinBlocks = 1; };
template <>
struct PairBudget<1> { static constexpr int kThreads = 128, kMinBlocks = 4; };
template <>
struct PairBudget<2> { static constexpr int kThreads = 128, kMinBlocks = 3; };

struct PairBufs {
    float* yhi;
    float* ylo;
    float* kacc;
};

template <int STAGE, class Acc>
struct PairSink {
    const Acc& A;
    const Layout& L;
    PairBufs b;
    float* __restrict__ xn;
    f2 h, w6;
    __device__ __forceinline__ static float2* at(float* base, int64_t q) { return reinterpret_cast<float2*>(base + q); }
    __device__ __forceinline__ static float2 rd(const float* base, int64_t q) {
        return __ldg(reinterpret_cast<const float2*>(base + q));
    }
    __device__ __forceinline__ void operator()(int a, f2 r) const {
        const int64_t q = a * L.P + A.c;
        if (STAGE == 1) {
            *at(b.kacc, q) = r.v;
            *at(xn, q) = (A.v(a) + h * r).v;
        } else if (STAGE < 4) {
            // read then written by this thread only: read-only path is safe
            *at(b.kacc, q) = (f2(rd(b.kacc, q)) + f2(2.f) * r).v;
            *at(xn, q) = (f2(rd(b.yhi, q)) + h * r).v;
        } else {
            const f2 s = f2(rd(b.kacc, q)) + r;
            f2 hi(rd(b.yhi, q)), lo(rd(b.ylo, q));
            acc_hilo(hi, lo, f2(w6 * s));
            *at(b.yhi, q) = hi.v;
            *at(b.ylo, q) = lo.v;
        }
    }
};

__device__ __forceinline__ void prefetch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// COMP: the compensated mode (gauge Laplacians and auxiliary gradients as
// compensated pairs, accessors.cuh PairAcc); scl = the coefficients' low parts.
template <int STAGE, bool BETA, int REG, bool COMP = false>
__global__ void __launch_bounds__(PairBudget<REG>::kThreads, PairBudget<REG>::kMinBlocks)
    k_stage_fp32x2(const __grid_constant__ Grid g, const __grid_constant__ Layout L, const __grid_constant__ Ptr36 X,
                   PairBufs b, float* __restrict__ xn, PhysCoef<f2> pc, StencilCoef<f2> sc, f2 h, f2 w6, int nbx,
                   int nby, int ycb, StencilCoef<f2> scl) {
    int bx, by, k;
    chunk_walk(blockIdx.x, nbx, nby, g.nz, ycb, bx, by, k);
    const int ip = bx * blockDim.x + threadIdx.x;  // pair index along x
    const int j = by * blockDim.y + threadIdx.y;
    const int i0 = 2 * ip;
    if (i0 >= g.nx || j >= g.ny) return;
    PairAcc<SrcPtr36<float>, COMP> A{{X}};
    A.place_ghost(i0, j, k, g.nx, L);
    A.s = sc;
    A.sl = scl;
    // L2 prefetch of this warp's lines of the epilogue operands (the RK4
    // accumulator and the state, read once each when the rates come out) and
    // of the stage input two planes up (read by the z stencils here and by
    // the blocks of the next planes).  The physics issues those loads late
    // and the warps wait on them.  Measured on GB300 at 256^3 with the 64x2
    // tile: 10.19 ms per step without, 9.75 with these prefetches; the stage
    // input at k+1 or k+3 instead of k+2: 9.80, at k+4: 9.91, two planes:
    // 10.02-10.15; the stage input alone (k+3): 9.96; the epilogue operands
    // alone: 3% slower than none.  Only full warps of one row prefetch: a
    // warp's 64 sites x 36 arrays are 72 lines of 128 bytes per buffer, two
    // or three per lane.  Plane k+2 <= nz+1 lies inside the ghosted box.
    if ((blockDim.x & 31) == 0 && i0 - 2 * (int)(threadIdx.x & 31) + 64 <= g.nx) {
        const int lane = threadIdx.x & 31;
        const int cw = A.c - 2 * lane;  // first site of the warp's 64-site segment
        const int kz = 2 * L.px * L.py;
        for (int q = lane; q < 72; q += 32) {
            const int64_t o = (q >> 1) * L.P + cw + 32 * (q & 1);
            if (STAGE > 1) {
                prefetch_l2(b.kacc + o);
                prefetch_l2(b.yhi + o);
            }
            if (STAGE == 4) prefetch_l2(b.ylo + o);
            prefetch_l2(reinterpret_cast<const float*>(X.p[q >> 1]) + cw + kz + 32 * (q & 1));
        }
    }
    PairSink<STAGE, PairAcc<SrcPtr36<float>, COMP>> out{A, L, b, xn, h, w6};
    site_rates<f2, BETA>(A, pc, out);
}

Ptr36 pack4(const void* base, int64_t S) {
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = static_cast<const char*>(base) + (size_t)a * S * 4;
    return P;
}

template <bool BETA, int REG, bool COMP = false>
void step_pair(const Grid& g, const Layout& L, const Tiling& t, PairBufs b, float* xa, float* xb,
               const PhysCoef<f2>& pc, const StencilCoef<f2>& sc, const StencilCoef<f2>& scl, double dt,
               cudaStream_t st) {
    const int npx = g.nx / 2;
    const int nbx = (npx + t.bx - 1) / t.bx, nby = (g.ny + t.by - 1) / t.by;
    const int ycb = std::max(1, kChunkRows / t.by);
    const dim3 gr(nbx * nby * g.nz), bl(t.bx, t.by);
    const f2 h2((float)(dt / 2.)), h1((float)dt), w6((float)(dt / 6.)), z(0.f);
#define EWPT_PAIR_ARGS nbx, nby, ycb, scl
    k_stage_fp32x2<1, BETA, REG, COMP><<<gr, bl, 0, st>>>(g, L, pack4(b.yhi, L.P), b, xa, pc, sc, h2, w6, EWPT_PAIR_ARGS);
    launch_ghost_fill(g, L, xa, st, false);
    k_stage_fp32x2<2, BETA, REG, COMP><<<gr, bl, 0, st>>>(g, L, pack4(xa, L.P), b, xb, pc, sc, h2, w6, EWPT_PAIR_ARGS);
    launch_ghost_fill(g, L, xb, st, false);
    k_stage_fp32x2<3, BETA, REG, COMP><<<gr, bl, 0, st>>>(g, L, pack4(xb, L.P), b, xa, pc, sc, h1, w6, EWPT_PAIR_ARGS);
    launch_ghost_fill(g, L, xa, st, false);
    k_stage_fp32x2<4, BETA, REG, COMP><<<gr, bl, 0, st>>>(g, L, pack4(xa, L.P), b, nullptr, pc, sc, z, w6, EWPT_PAIR_ARGS);
    launch_ghost_fill(g, L, b.yhi, st, false);
#undef EWPT_PAIR_ARGS
}

template <bool BETA>
void step_pair_r(const Grid& g, const Layout& L, const Tiling& t, PairBufs b, float* xa, float* xb,
                 const PhysCoef<f2>& pc, const StencilCoef<f2>& sc, const StencilCoef<f2>& scl, bool comp,
                 double dt, cudaStream_t st) {
    if (comp)  // one register budget (<= 168) for the compensated mode
        step_pair<BETA, 2, true>(g, L, t, b, xa, xb, pc, sc, scl, dt, st);
    else if (t.reg == 1)
        step_pair<BETA, 1>(g, L, t, b, xa, xb, pc, sc, scl, dt, st);
    else if (t.reg == 2)
        step_pair<BETA, 2>(g, L, t, b, xa, xb, pc, sc, scl, dt, st);
    else
        step_pair<BETA, 0>(g, L, t, b, xa, xb, pc, sc, scl, dt, st);
}

}  // namespace

cudaError_t launch_step_fp32_pair(const Grid& g, const Layout& L, const Tiling& t, Fp32State y, Fp32Work w,
                                  const ewpt_params& p, double Jex, double gam, cudaStream_t st, bool comp) {
    if (g.nx % 2 != 0 || L.gx == 0) return cudaErrorInvalidValue;
    const PhysCoef<f2> pc = make_phys<f2>(p, Jex, gam);
    const StencilCoef<f2> sc = pair_stencil(make_stencil<float>(p.dx));
    const StencilCoef<f2> scl = pair_stencil_lo(make_stencil<double>(p.dx));
    PairBufs b{y.hi, y.lo, w.kacc};
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        step_pair_r<true>(g, L, t, b, w.xa, w.xb, pc, sc, scl, comp, p.dt, st);
    else
        step_pair_r<false>(g, L, t, b, w.xa, w.xb, pc, sc, scl, comp, p.dt, st);
    return cudaGetLastError();
}
