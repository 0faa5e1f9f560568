// stage_dd.cu -- DF64 form: the FP64 form's stage kernels (stage.cu) with
// every stencil, flux and RK4 combination evaluated in double-float
// arithmetic (dd.cuh) on the FP32 pipes.
//
// The state, the RK4 accumulator and the stage inputs keep the FP64 form's
// buffers and scheme (y, yn, xa, xb, [36][S] of 8 bytes, the reference's
// yn accumulation order, main_rk4.jl:6146-6437), each value stored as the
// float pair (hi, lo).  State I/O converts from / to FP64 exactly
// representable splits (hi = fl(v), lo = fl(v - hi)).
#include "accessors.cuh"
#include "dd.cuh"

namespace {

template <int REG>
struct DdBudget;
template <>
struct DdBudget<0> { static constexpr int kThreads = 128, kMinBlocks = 1; };
template <>
struct DdBudget<2> { static constexpr int kThreads = 128, kMinBlocks = 3; };

// Stencil sums in double-float with lazy normalisation: each partial sum is
// an unnormalised pair (h, l), h + l the value, |l| a few ulp of h at most.
// An addition is Knuth's TwoSum on the high parts plus the low parts (8
// FP32 operations); a product by a coefficient is the FMA product error
// plus the cross terms (4).  Only a finished derivative is renormalised
// (FastTwoSum, 3), where dd's operators renormalise after every operation
// (11 and 7).  The error per operation stays ~2^-47 of the operands.
struct Lz {
    float h, l;
};
__device__ __forceinline__ Lz lz_add(const Lz& a, const Lz& b) {
    const float s = a.h + b.h;
    const float v = s - a.h;
    const float e = (a.h - (s - v)) + (b.h - v);
    return Lz{s, e + (a.l + b.l)};
}
__device__ __forceinline__ Lz lz_sub(const Lz& a, const Lz& b) { return lz_add(a, Lz{-b.h, -b.l}); }
__device__ __forceinline__ Lz lz_mul(const dd& c, const Lz& x) {
    const float p = c.hi * x.h;
    float e = fmaf(c.hi, x.h, -p);
    e = fmaf(c.hi, x.l, e);
    e = fmaf(c.lo, x.h, e);
    return Lz{p, e};
}
__device__ __forceinline__ dd lz_done(const Lz& x) { return dd_fast_two_sum(x.h, x.l); }

// The stencil evaluations are out-of-line calls: the double-float stage is
// instruction-fetch bound (~20 k straight-line instructions per site), and
// one copy of each stencil routine replaces 16 + 4 + 4 inlined copies.
struct DdAcc : SiteAcc<float2, dd, SrcPtr36<float2>> {
    using Base = SiteAcc<float2, dd, SrcPtr36<float2>>;
    __device__ __forceinline__ Lz lz(int a, int off) const {
        const float2 v = __ldg(src.arr(a) + (c + off));
        return Lz{v.x, v.y};
    }
    // derivative along one axis (offsets o) in unnormalised form
    __device__ __forceinline__ Lz d1_lz(int a, const int* o) const {
        Lz g = lz_mul(s.a1, lz_sub(lz(a, o[0]), lz(a, o[3])));
        g = lz_add(g, lz_mul(s.a2, lz_sub(lz(a, o[1]), lz(a, o[4]))));
        return lz_add(g, lz_mul(s.a3, lz_sub(lz(a, o[2]), lz(a, o[5]))));
    }
    __device__ __noinline__ void grad_lap(int a, dd& gx, dd& gy, dd& gz, dd& lap) const {
        Lz S[3];  // sum over the axes of f(+k) + f(-k), k = 1, 2, 3
        const int* os[3] = {ox, oy, oz};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int* o = os[ax];
            Lz g;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const Lz p = lz(a, o[k]), m = lz(a, o[k + 3]);
                const dd& ck = k == 0 ? s.a1 : (k == 1 ? s.a2 : s.a3);
                const Lz t = lz_mul(ck, lz_sub(p, m));
                g = k == 0 ? t : lz_add(g, t);
                const Lz q = lz_add(p, m);
                S[k] = ax == 0 ? q : lz_add(S[k], q);
            }
            (ax == 0 ? gx : (ax == 1 ? gy : gz)) = lz_done(g);
        }
        Lz L = lz_mul(s.l0, lz(a, 0));
        L = lz_add(L, lz_mul(s.l1, S[0]));
        L = lz_add(L, lz_mul(s.l2, S[1]));
        lap = lz_done(lz_add(L, lz_mul(s.l3, S[2])));
    }
    __device__ __noinline__ void grad(int a, dd& gx, dd& gy, dd& gz) const {
        gx = lz_done(d1_lz(a, ox));
        gy = lz_done(d1_lz(a, oy));
        gz = lz_done(d1_lz(a, oz));
    }
    __device__ __noinline__ dd div3(int a) const {
        return lz_done(lz_add(lz_add(d1_lz(a, ox), d1_lz(a + 1, oy)), d1_lz(a + 2, oz)));
    }
};

template <int STAGE>
struct DdSink {
    const DdAcc& A;
    const float2* __restrict__ y;
    float2* yn;
    float2* __restrict__ xn;
    float2* acc_out;
    int64_t S;
    dd w, h;
    float2* cur;  // [12][S] Higgs currents of kt W and kt Y, from the first launch of a split stage to the others
    __device__ __forceinline__ void keep_current(int q, dd v) const { cur[q * S + A.c] = v.f2(); }
    __device__ __forceinline__ dd load_current(int q) const { return dd(__ldg(cur + q * S + A.c)); }
    __device__ __forceinline__ void operator()(int a, dd r) const {
        const int64_t q = a * S + A.c;
        if (STAGE == 1) {
            const dd ya = A.v(a);  // X1 == y
            yn[q] = (ya + w * r).f2();
            xn[q] = (ya + h * r).f2();
        } else if (STAGE < 4) {
            // read then written by this thread only: read-only path is safe
            yn[q] = (dd(__ldg(yn + q)) + w * r).f2();
            xn[q] = (dd(__ldg(y + q)) + h * r).f2();
        } else {
            acc_out[q] = (dd(__ldg(yn + q)) + w * r).f2();
        }
    }
};

Ptr36 pack8(const void* base, int64_t S) {
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = static_cast<const char*>(base) + (size_t)a * S * 8;
    return P;
}

// PART (site_rates): 0 the whole stage; 1-3 its three parts (Higgs; SU(2);
// fields, auxiliaries and U(1)), launched one after the other when there
// are no beta terms.  The double-float stage is instruction-fetch bound
// (~20 k straight-line instructions per site): each part is a third of the
// code, and the stencil routines are shared out-of-line calls.
template <int STAGE, bool BETA, int REG, int PART>
__global__ void __launch_bounds__(DdBudget<REG>::kThreads, DdBudget<REG>::kMinBlocks)
    k_stage_dd(Grid g, const __grid_constant__ Ptr36 X, const float2* __restrict__ y, float2* yn,
               float2* __restrict__ xn, float2* acc_out, PhysCoef<dd> pc, StencilCoef<dd> sc, dd w, dd h,
               float2* cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    DdAcc A{{{X}}};
    A.place(i, j, k, g.nx, g.ny, g.nz);
    A.s = sc;
    DdSink<STAGE> out{A, y, yn, xn, acc_out, g.S, w, h, cur};
    site_rates<dd, BETA, DdAcc, DdSink<STAGE>, PART>(A, pc, out);
}

__global__ void k_to_dd(int64_t n, double* __restrict__ v) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        reinterpret_cast<float2*>(v)[q] = dd(v[q]).f2();
}

__global__ void k_from_dd(int64_t n, const double* __restrict__ src, double* __restrict__ dst) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2*>(src)[q];
        dst[q] = (double)v.x + (double)v.y;
    }
}


// One stage: the whole stage with beta terms, else its three parts.
template <int STAGE, bool BETA, int REG>
void stage_dd(const dim3& gr, const dim3& bl, cudaStream_t st, const Grid& g, const float2* X, const float2* y,
              float2* yn, float2* xn, float2* acc_out, const PhysCoef<dd>& pc, const StencilCoef<dd>& sc, dd w,
              dd h, float2* cur) {
    const Ptr36 P = pack8(X, g.S);
    if constexpr (BETA) {
        k_stage_dd<STAGE, true, REG, 0><<<gr, bl, 0, st>>>(g, P, y, yn, xn, acc_out, pc, sc, w, h, cur);
    } else {
        k_stage_dd<STAGE, false, REG, 1><<<gr, bl, 0, st>>>(g, P, y, yn, xn, acc_out, pc, sc, w, h, cur);
        k_stage_dd<STAGE, false, REG, 2><<<gr, bl, 0, st>>>(g, P, y, yn, xn, acc_out, pc, sc, w, h, cur);
        k_stage_dd<STAGE, false, REG, 3><<<gr, bl, 0, st>>>(g, P, y, yn, xn, acc_out, pc, sc, w, h, cur);
    }
}

template <bool BETA, int REG>
void step_dd(const Grid& g, const Tiling& t, float2* y, float2* yn, float2* xa, float2* xb, const PhysCoef<dd>& pc,
             const StencilCoef<dd>& sc, double dt, float2* cur, cudaStream_t st) {
    const dim3 gr((g.nx + t.bx - 1) / t.bx, (g.ny + t.by - 1) / t.by, g.nz), bl(t.bx, t.by);
    const dd w6(dt / 6.), w3(dt / 3.), h2(dt / 2.), h1(dt), z(0.0);
    stage_dd<1, BETA, REG>(gr, bl, st, g, y, y, yn, xa, nullptr, pc, sc, w6, h2, cur);
    stage_dd<2, BETA, REG>(gr, bl, st, g, xa, y, yn, xb, nullptr, pc, sc, w3, h2, cur);
    stage_dd<3, BETA, REG>(gr, bl, st, g, xb, y, yn, xa, nullptr, pc, sc, w3, h1, cur);
    stage_dd<4, BETA, REG>(gr, bl, st, g, xa, y, yn, nullptr, y, pc, sc, w6, z, cur);
}

template <bool BETA>
void step_dd_r(const Grid& g, const Tiling& t, float2* y, float2* yn, float2* xa, float2* xb, const PhysCoef<dd>& pc,
               const StencilCoef<dd>& sc, double dt, float2* cur, cudaStream_t st) {
    // the 128-register variant spills heavily in this form and runs as variant 0
    if (t.reg == 2)
        step_dd<BETA, 2>(g, t, y, yn, xa, xb, pc, sc, dt, cur, st);
    else
        step_dd<BETA, 0>(g, t, y, yn, xa, xb, pc, sc, dt, cur, st);
}

}  // namespace

cudaError_t launch_step_dd(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                           double* cur, const ewpt_params& p, double Jex, double gam, cudaStream_t st) {
    const PhysCoef<dd> pc = make_phys<dd>(p, Jex, gam);
    const StencilCoef<dd> sc = make_stencil<dd>(p.dx);
    auto f2p = [](double* v) { return reinterpret_cast<float2*>(v); };
    if (p.beta_w != 0.0 || p.beta_y != 0.0)
        step_dd_r<true>(g, t, f2p(y), f2p(yn), f2p(xa), f2p(xb), pc, sc, p.dt, f2p(cur), st);
    else
        step_dd_r<false>(g, t, f2p(y), f2p(yn), f2p(xa), f2p(xb), pc, sc, p.dt, f2p(cur), st);
    return cudaGetLastError();
}

cudaError_t launch_to_dd(int64_t n, double* v, cudaStream_t st) {
    k_to_dd<<<1216, 256, 0, st>>>(n, v);
    return cudaGetLastError();
}

cudaError_t launch_from_dd(int64_t n, const double* src, double* dst, cudaStream_t st) {
    k_from_dd<<<1216, 256, 0, st>>>(n, src, dst);
    return cudaGetLastError();
}
