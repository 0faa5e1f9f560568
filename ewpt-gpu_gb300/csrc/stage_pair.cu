// stage_pair.cu -- FP32-form RK4 stage kernels with two sites per thread.
//
// Same stage structure and arithmetic as k_stage_fp32 (stage.cu), but each
// thread owns the x-adjacent sites (i0, i0+1), i0 even, and runs the physics
// on packed float pairs (f32x2.cuh): every flux operation is one FFMA2 /
// FADD2 / FMUL2 for both sites, and every neighbour access is a float2 load.
// For the x stencil the pairs at i0-4, i0-2, i0, i0+2, i0+4 (five aligned
// float2 loads) are re-paired into the +-1, +-2, +-3 neighbour pairs; y and z
// neighbours are aligned float2 loads of the same x pair.  Needs nx even
// (a pair never straddles the periodic wrap).
#include "ewpt_internal.cuh"
#include "f32x2.cuh"

namespace {

template <int REG>
struct PairBudget;
template <>
struct PairBudget<0> { static constexpr int kThreads = 128, kMinBlocks = 1; };
template <>
struct PairBudget<1> { static constexpr int kThreads = 128, kMinBlocks = 4; };
template <>
struct PairBudget<2> { static constexpr int kThreads = 128, kMinBlocks = 3; };

struct PairAcc {
    const Ptr36& P;
    int c;        // linear index of site i0 (even)
    int ox[4];    // float offsets of the x pairs at i0-4, i0-2, i0+2, i0+4 (wrapped)
    int oy[6], oz[6];
    StencilCoef<f2> s;

    __device__ __forceinline__ float2 ld(int a, int off) const {
        return __ldg(reinterpret_cast<const float2*>(reinterpret_cast<const float*>(P.p[a]) + (c + off)));
    }
    __device__ __forceinline__ f2 v(int a) const { return f2(ld(a, 0)); }
    // x-neighbour pairs of the two sites: p1 = (f[i0+1], f[i0+2]) ... m3 = (f[i0-3], f[i0-2])
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
            if (ax == 0) gy = g; else gz = g;
            s1 += p1 + m1;
            s2 += p2 + m2;
            s3 += p3 + m3;
        }
        lap = s.l0 * v(a) + s.l1 * s1 + s.l2 * s2 + s.l3 * s3;
    }
    __device__ __forceinline__ f2 div3(int a) const { return dx(a) + d1(a + 1, oy) + d1(a + 2, oz); }
};

// Compensated accumulation on both lanes (TwoSum, then renormalise).
__device__ __forceinline__ void acc2x2(f2& hi, f2& lo, f2 p) {
    const f2 s = hi + p;
    const f2 bp = s - hi;
    const f2 e = (hi - (s - bp)) + (p - bp);
    const f2 t = lo + e;
    hi = s + t;
    lo = t - (hi - s);
}

struct PairBufs {
    float* yhi;
    float* ylo;
    float* kacc;
};

template <int STAGE>
struct PairSink {
    const PairAcc& A;
    PairBufs b;
    float* __restrict__ xn;
    int64_t S;
    f2 h, w6;
    __device__ __forceinline__ static float2* at(float* base, int64_t q) { return reinterpret_cast<float2*>(base + q); }
    __device__ __forceinline__ static float2 rd(const float* base, int64_t q) {
        return __ldg(reinterpret_cast<const float2*>(base + q));
    }
    __device__ __forceinline__ void operator()(int a, f2 r) const {
        const int64_t q = a * S + A.c;
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
            acc2x2(hi, lo, f2(w6 * s));
            *at(b.yhi, q) = hi.v;
            *at(b.ylo, q) = lo.v;
        }
    }
};

template <int STAGE, bool BETA, int REG>
__global__ void __launch_bounds__(PairBudget<REG>::kThreads, PairBudget<REG>::kMinBlocks)
    k_stage_fp32x2(Grid g, const __grid_constant__ Ptr36 X, PairBufs b, float* __restrict__ xn,
                   PhysCoef<f2> pc, StencilCoef<f2> sc, f2 h, f2 w6) {
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;  // pair index along x
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int i0 = 2 * ip;
    if (i0 >= g.nx || j >= g.ny) return;
    PairAcc A{X};
    A.c = i0 + g.nx * (j + g.ny * k);
    A.ox[0] = (i0 - 4 >= 0 ? -4 : g.nx - 4);
    A.ox[1] = (i0 - 2 >= 0 ? -2 : g.nx - 2);
    A.ox[2] = (i0 + 2 < g.nx ? 2 : 2 - g.nx);
    A.ox[3] = (i0 + 4 < g.nx ? 4 : 4 - g.nx);
    axis_offsets(j, g.ny, g.nx, A.oy);
    axis_offsets(k, g.nz, g.nx * g.ny, A.oz);
    A.s = sc;
    PairSink<STAGE> out{A, b, xn, g.S, h, w6};
    site_rates<f2, BETA>(A, pc, out);
}

template <typename T>
StencilCoef<f2> pair_stencil(const StencilCoef<T>& s) {
    return StencilCoef<f2>{f2(s.a1), f2(s.a2), f2(s.a3), f2(s.l0), f2(s.l1), f2(s.l2), f2(s.l3)};
}

Ptr36 pack4(const void* base, int64_t S) {
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = static_cast<const char*>(base) + (size_t)a * S * 4;
    return P;
}

template <bool BETA, int REG>
void step_pair(const Grid& g, const Tiling& t, PairBufs b, float* xa, float* xb, const PhysCoef<f2>& pc,
               const StencilCoef<f2>& sc, double dt, cudaStream_t st) {
    const int npx = g.nx / 2;
    const dim3 gr((npx + t.bx - 1) / t.bx, (g.ny + t.by - 1) / t.by, g.nz), bl(t.bx, t.by);
    const f2 h2((float)(dt / 2.)), h1((float)dt), w6((float)(dt / 6.)), z(0.f);
    k_stage_fp32x2<1, BETA, REG><<<gr, bl, 0, st>>>(g, pack4(b.yhi, g.S), b, xa, pc, sc, h2, w6);
    k_stage_fp32x2<2, BETA, REG><<<gr, bl, 0, st>>>(g, pack4(xa, g.S), b, xb, pc, sc, h2, w6);
    k_stage_fp32x2<3, BETA, REG><<<gr, bl, 0, st>>>(g, pack4(xb, g.S), b, xa, pc, sc, h1, w6);
    k_stage_fp32x2<4, BETA, REG><<<gr, bl, 0, st>>>(g, pack4(xa, g.S), b, nullptr, pc, sc, z, w6);
}

template <bool BETA>
void step_pair_r(const Grid& g, const Tiling& t, PairBufs b, float* xa, float* xb, const PhysCoef<f2>& pc,
                 const StencilCoef<f2>& sc, double dt, cudaStream_t st) {
    if (t.reg == 1)
        step_pair<BETA, 1>(g, t, b, xa, xb, pc, sc, dt, st);
    else if (t.reg == 2)
        step_pair<BETA, 2>(g, t, b, xa, xb, pc, sc, dt, st);
    else
        step_pair<BETA, 0>(g, t, b, xa, xb, pc, sc, dt, st);
}

}  // namespace

cudaError_t launch_step_fp32_pair(const Grid& g, const Tiling& t, Fp32State y, Fp32Work w, const ewpt_params& p,
                                  double Jex, double gam, cudaStream_t st) {
    if (g.nx % 2 != 0) return cudaErrorInvalidValue;
    const PhysCoef<f2> pc = make_phys<f2>(p, Jex, gam);
    const StencilCoef<f2> sc = pair_stencil(make_stencil<float>(p.dx));
    PairBufs b{y.hi, y.lo, w.kacc};
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        step_pair_r<true>(g, t, b, w.xa, w.xb, pc, sc, p.dt, st);
    else
        step_pair_r<false>(g, t, b, w.xa, w.xb, pc, sc, p.dt, st);
    return cudaGetLastError();
}
