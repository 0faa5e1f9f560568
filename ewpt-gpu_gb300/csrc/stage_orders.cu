// stage_orders.cu -- FP64 stage and rate kernels with the alternative
// stencil orders (2nd, 8th, 10th, 12th; stencil_n.cuh).
//
// Same physics (physics.cuh) and RK4 scheme as the 6th-order FP64 kernels of
// stage.cu (the reference's yn accumulation order, main_rk4.jl:6146-6437);
// only the accessor changes.  One register-budget variant (compiler's
// choice) per order.
#include "accessors.cuh"
#include "stencil_n.cuh"

namespace {

template <int R>
using AccN = SiteAccN<double, double, SrcPtr36<double>, R>;

template <int STAGE, int R>
struct SinkN {
    const AccN<R>& A;
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
            // read then written by this thread only: read-only path is safe
            yn[q] = fma(r, w, __ldg(yn + q));
            xn[q] = fma(r, h, __ldg(y + q));
        } else {
            acc_out[q] = fma(r, w, __ldg(yn + q));
        }
    }
};

template <int R>
__device__ __forceinline__ bool place_n(const Grid& g, const StencilN<double, R>& sc, AccN<R>& A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return false;
    A.place(i, j, blockIdx.z, g.nx, g.ny, g.nz);
    A.s = sc;
    return true;
}

template <int STAGE, bool BETA, int R>
__global__ void __launch_bounds__(128, 1)
    k_stage_fp64n(Grid g, const __grid_constant__ Ptr36 X, const double* __restrict__ y, double* yn,
                  double* __restrict__ xn, double* acc_out, PhysCoef<double> pc, StencilN<double, R> sc, double w,
                  double h) {
    AccN<R> A{{X}};
    if (!place_n(g, sc, A)) return;
    SinkN<STAGE, R> out{A, y, yn, xn, acc_out, g.S, w, h};
    site_rates<double, BETA>(A, pc, out);
}

struct RatesSinkN {
    const MPtr36& Rr;
    int c;
    __device__ __forceinline__ void operator()(int a, double r) const { reinterpret_cast<double*>(Rr.p[a])[c] = r; }
};

template <bool BETA, int R>
__global__ void __launch_bounds__(128, 1) k_rates_fp64n(Grid g, const __grid_constant__ Ptr36 X,
                                                         const __grid_constant__ MPtr36 Rr, PhysCoef<double> pc,
                                                         StencilN<double, R> sc) {
    AccN<R> A{{X}};
    if (!place_n(g, sc, A)) return;
    RatesSinkN out{Rr, A.c};
    site_rates<double, BETA>(A, pc, out);
}

Ptr36 pack_d(const void* base, int64_t S) {
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = static_cast<const char*>(base) + (size_t)a * S * 8;
    return P;
}

dim3 grid_n(const Grid& g, int bx, int by) { return dim3((g.nx + bx - 1) / bx, (g.ny + by - 1) / by, g.nz); }

template <bool BETA, int R>
void step_n(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb, const PhysCoef<double>& pc,
            double dx, double dt, cudaStream_t st) {
    const StencilN<double, R> sc = make_stencil_n<double, R>(dx);
    const dim3 gr = grid_n(g, t.bx, t.by), bl(t.bx, t.by);
    k_stage_fp64n<1, BETA, R><<<gr, bl, 0, st>>>(g, pack_d(y, g.S), y, yn, xa, nullptr, pc, sc, dt / 6., dt / 2.);
    k_stage_fp64n<2, BETA, R><<<gr, bl, 0, st>>>(g, pack_d(xa, g.S), y, yn, xb, nullptr, pc, sc, dt / 3., dt / 2.);
    k_stage_fp64n<3, BETA, R><<<gr, bl, 0, st>>>(g, pack_d(xb, g.S), y, yn, xa, nullptr, pc, sc, dt / 3., dt);
    k_stage_fp64n<4, BETA, R><<<gr, bl, 0, st>>>(g, pack_d(xa, g.S), y, yn, nullptr, y, pc, sc, dt / 6., 0.0);
}

template <int R>
void step_nb(bool beta, const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
             const PhysCoef<double>& pc, double dx, double dt, cudaStream_t st) {
    if (beta)
        step_n<true, R>(g, t, y, yn, xa, xb, pc, dx, dt, st);
    else
        step_n<false, R>(g, t, y, yn, xa, xb, pc, dx, dt, st);
}

template <int R>
void rates_nb(bool beta, const Grid& g, const Ptr36& in, const MPtr36& out, const PhysCoef<double>& pc, double dx,
              cudaStream_t st) {
    const StencilN<double, R> sc = make_stencil_n<double, R>(dx);
    if (beta)
        k_rates_fp64n<true, R><<<grid_n(g, 32, 4), dim3(32, 4), 0, st>>>(g, in, out, pc, sc);
    else
        k_rates_fp64n<false, R><<<grid_n(g, 32, 4), dim3(32, 4), 0, st>>>(g, in, out, pc, sc);
}

}  // namespace

cudaError_t launch_step_fp64_order(const Grid& g, const Tiling& t, double* y, double* yn, double* xa, double* xb,
                                   const ewpt_params& p, double Jex, double gam, cudaStream_t st) {
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const bool beta = p.beta_w != 0.0 || p.beta_y != 0.0;
    const Tiling tt{t.bx, t.by, 0, 0};
    switch (stencil_radius(p.stencil_order)) {
        case 1: step_nb<1>(beta, g, tt, y, yn, xa, xb, pc, p.dx, p.dt, st); break;
        case 4: step_nb<4>(beta, g, tt, y, yn, xa, xb, pc, p.dx, p.dt, st); break;
        case 5: step_nb<5>(beta, g, tt, y, yn, xa, xb, pc, p.dx, p.dt, st); break;
        case 6: step_nb<6>(beta, g, tt, y, yn, xa, xb, pc, p.dx, p.dt, st); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_rates_fp64_order(const Grid& g, const Ptr36& in, const MPtr36& out, const ewpt_params& p,
                                    double Jex, double gam, cudaStream_t st) {
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const bool beta = p.beta_w != 0.0 || p.beta_y != 0.0;
    switch (stencil_radius(p.stencil_order)) {
        case 1: rates_nb<1>(beta, g, in, out, pc, p.dx, st); break;
        case 4: rates_nb<4>(beta, g, in, out, pc, p.dx, st); break;
        case 5: rates_nb<5>(beta, g, in, out, pc, p.dx, st); break;
        case 6: rates_nb<6>(beta, g, in, out, pc, p.dx, st); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
