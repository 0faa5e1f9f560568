// thermal.cu -- thermal initial condition generated on the device.
//
// The construction of the reference's thermal initializer
// (thermal_initializer_phi! / thermal_initializer_gauge!,
// main_rk4.jl:5029-5152, driven from :5348-5636): every field is
// real(bfft(z)) of a spectrum z(k) = amp(k) (a + i b) with a, b ~ N(0, sqrt 2)
// per mode, amp = sqrt(n(w) / (w V)) and the Bose-Einstein occupation
// n(w) = 1 / (exp(w / T) - 1), k^2 = sum_i 2 (1 - cos theta_i) / dx^2.
//   Higgs phi_1..4   w^2 = k^2 + mH^2, one scalar spectrum per component;
//   W^a_i, Y_i       two transverse polarisations: e1 = r x k / |r x k| with
//                    r ~ N(0, sqrt 2)^3, e2 = e1 x k / |e1 x k|, k the lattice
//                    momentum 2 sin(theta / 2) / dx; z_i = amp (e1_i (x1 + i x3)
//                    + e2_i (x2 + i x4)); w^2 = k^2 + mW^2 for W, k^2 for Y;
//                    the k = 0 mode is left empty;
//   Gamma^a, Sigma   the divergence of W^a and Y with the context's stencil,
//                    so that the auxiliary constraints hold at t = 0;
//   momenta          zero, as in the reference.
// The mode index n is the FFT index wrapped to [-N/2, N/2) (theta = 2 pi n / N).
// The same construction runs on the host in ewpt/ic.py (thermal, with
// with_momenta=False); the random numbers differ: here each deviate is a
// counter-based hash of (seed, stream, mode) -- SplitMix64 (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", 2014) -- turned
// into normals by the Box-Muller transform, so a state is reproducible from
// its seed on any GPU and at any launch shape.
#include <cufft.h>

#include <cmath>
#include <string>

#include "ewpt_ctx.cuh"
#include "stencil_n.cuh"

namespace {

constexpr double kTwoPi = 6.283185307179586;

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Two N(0, sqrt 2) deviates of draw `stream` at mode q.
__device__ __forceinline__ void normal_pair(uint64_t key, int stream, int64_t q, double& a, double& b) {
    const uint64_t k = splitmix64(key ^ splitmix64(0x51ED270B27A3C4F1ull * (uint64_t)(stream + 1)));
    const uint64_t h1 = splitmix64(k ^ (2 * (uint64_t)q)), h2 = splitmix64(k ^ (2 * (uint64_t)q + 1));
    const double u1 = ((double)(h1 >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
    const double u2 = (double)(h2 >> 11) * 0x1.0p-53;          // [0, 1)
    const double r = sqrt(-4.0 * log(u1));                      // sqrt 2 * sqrt(-2 log u1)
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    a = r * c;
    b = r * s;
}

struct ModeGeom {
    double k2;        // lattice k^2
    double kv[3];     // lattice momentum 2 sin(theta / 2) / dx
};

// Mode q of the spectrum array: theta = 2 pi n / N per axis with n the FFT
// index wrapped to [-N/2, N/2), or, with one_based, the reference's 1-based
// array index (n = index + 1: the element bfft treats as frequency f gets
// the amplitude of frequency f + 1, main_rk4.jl:5040-5046).
__device__ __forceinline__ ModeGeom mode_geom(const Grid& g, double dx, int64_t q, bool one_based = false) {
    const int i = (int)(q % g.nx), j = (int)((q / g.nx) % g.ny), k = (int)(q / ((int64_t)g.nx * g.ny));
    int n[3] = {i < (g.nx + 1) / 2 ? i : i - g.nx, j < (g.ny + 1) / 2 ? j : j - g.ny,
                k < (g.nz + 1) / 2 ? k : k - g.nz};
    if (one_based) {
        n[0] = i + 1;
        n[1] = j + 1;
        n[2] = k + 1;
    }
    const int N[3] = {g.nx, g.ny, g.nz};
    ModeGeom m;
    m.k2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double th = kTwoPi * n[d] / N[d];
        m.k2 += 2.0 * (1.0 - cos(th)) / (dx * dx);
        m.kv[d] = 2.0 * sin(0.5 * th) / dx;
    }
    return m;
}

__device__ __forceinline__ double occupation(double w, double T) { return w > 0.0 ? 1.0 / expm1(w / T) : 0.0; }

// amp(k) = sqrt(n(w) / (w V)) for a field, sqrt(n(w) w / V) for its momentum
// (mom), w^2 = k^2 + m^2; zero at k = 0 when empty_k0.
__device__ __forceinline__ double amplitude(double k2, double m, double T, double vol, bool empty_k0,
                                            bool mom = false) {
    if (empty_k0 && k2 == 0.0) return 0.0;
    const double w = sqrt(k2 + m * m);
    if (!(w > 0.0)) return 0.0;
    return mom ? sqrt(occupation(w, T) * w / vol) : sqrt(occupation(w, T) / (w * vol));
}

__global__ void k_modes_scalar(Grid g, double dx, double T, double m, double vol, uint64_t key, int stream,
                               cufftDoubleComplex* __restrict__ z, int mom) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const ModeGeom mg = mode_geom(g, dx, q);
        const double amp = amplitude(mg.k2, m, T, vol, false, mom != 0);
        double a, b;
        normal_pair(key, stream, q, a, b);
        z[q] = make_cuDoubleComplex(amp * a, amp * b);
    }
}

__global__ void k_modes_transverse(Grid g, double dx, double T, double m, double vol, uint64_t key, int stream,
                                   cufftDoubleComplex* __restrict__ z0, cufftDoubleComplex* __restrict__ z1,
                                   cufftDoubleComplex* __restrict__ z2, int mom) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const ModeGeom mg = mode_geom(g, dx, q);
        const double* kv = mg.kv;
        double r[4], x[4];
        normal_pair(key, stream, q, r[0], r[1]);
        normal_pair(key, stream + 1, q, r[2], r[3]);
        normal_pair(key, stream + 2, q, x[0], x[1]);
        normal_pair(key, stream + 3, q, x[2], x[3]);
        double e1[3] = {r[1] * kv[2] - r[2] * kv[1], r[2] * kv[0] - r[0] * kv[2], r[0] * kv[1] - r[1] * kv[0]};
        double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        n1 = n1 == 0.0 ? 1.0 : n1;
        for (int d = 0; d < 3; ++d) e1[d] /= n1;
        double e2[3] = {e1[1] * kv[2] - e1[2] * kv[1], e1[2] * kv[0] - e1[0] * kv[2], e1[0] * kv[1] - e1[1] * kv[0]};
        double n2 = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
        n2 = n2 == 0.0 ? 1.0 : n2;
        for (int d = 0; d < 3; ++d) e2[d] /= n2;
        const double amp = amplitude(mg.k2, m, T, vol, true, mom != 0);
        // x1 + i x3 on e1, x2 + i x4 on e2 (thermal_initializer_gauge!)
        cufftDoubleComplex* out[3] = {z0, z1, z2};
#pragma unroll
        for (int d = 0; d < 3; ++d)
            out[d][q] = make_cuDoubleComplex(amp * (e1[d] * x[0] + e2[d] * x[1]), amp * (e1[d] * x[2] + e2[d] * x[3]));
    }
}

// The same spectra from caller-supplied deviates, as the reference's own
// kernels scale them (thermal_initializer_phi!, thermal_initializer_gauge!,
// main_rk4.jl:5029-5152): one real deviate per Higgs mode; for a gauge field
// the arrays r_1 r_2 r_3 (the polarisation draw), r_1_i r_2_i r_3_i (unused,
// overwritten by the reference), x_1 x_2 x_3 x_4 at d[0..9] S apart.
__global__ void k_dev_scalar(Grid g, double dx, double T, double m, double vol, int one_based,
                             const double* __restrict__ d, cufftDoubleComplex* __restrict__ z) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const ModeGeom mg = mode_geom(g, dx, q, one_based);
        z[q] = make_cuDoubleComplex(amplitude(mg.k2, m, T, vol, false) * d[q], 0.0);
    }
}

__global__ void k_dev_transverse(Grid g, double dx, double T, double m, double vol, int one_based,
                                 const double* __restrict__ d, cufftDoubleComplex* __restrict__ z0,
                                 cufftDoubleComplex* __restrict__ z1, cufftDoubleComplex* __restrict__ z2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const ModeGeom mg = mode_geom(g, dx, q, one_based);
        const double* kv = mg.kv;
        const double r[3] = {d[q], d[g.S + q], d[2 * g.S + q]};
        const double x[4] = {d[6 * g.S + q], d[7 * g.S + q], d[8 * g.S + q], d[9 * g.S + q]};
        double e1[3] = {r[1] * kv[2] - r[2] * kv[1], r[2] * kv[0] - r[0] * kv[2], r[0] * kv[1] - r[1] * kv[0]};
        double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        n1 = n1 == 0.0 ? 1.0 : n1;
        for (int c = 0; c < 3; ++c) e1[c] /= n1;
        double e2[3] = {e1[1] * kv[2] - e1[2] * kv[1], e1[2] * kv[0] - e1[0] * kv[2], e1[0] * kv[1] - e1[1] * kv[0]};
        double n2 = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
        n2 = n2 == 0.0 ? 1.0 : n2;
        for (int c = 0; c < 3; ++c) e2[c] /= n2;
        const double amp = amplitude(mg.k2, m, T, vol, true);
        cufftDoubleComplex* out[3] = {z0, z1, z2};
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[c][q] = make_cuDoubleComplex(amp * (e1[c] * x[0] + e2[c] * x[1]), amp * (e1[c] * x[2] + e2[c] * x[3]));
    }
}

__global__ void k_real_part(int64_t S, const cufftDoubleComplex* __restrict__ z, double* __restrict__ f) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < S; q += (int64_t)gridDim.x * blockDim.x)
        f[q] = cuCreal(z[q]);
}

// div[b] = sum_i d_i f[3 b + i] for b < nb, periodic stencil of radius R.
template <int R>
__global__ void k_divergence(Grid g, StencilN<double, R> s, const double* __restrict__ f, int nb, double* __restrict__ div) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % g.nx), j = (int)((q / g.nx) % g.ny), k = (int)(q / ((int64_t)g.nx * g.ny));
        int o[3][2 * R];
        axis_offsets_n<R>(i, g.nx, 1, o[0]);
        axis_offsets_n<R>(j, g.ny, g.nx, o[1]);
        axis_offsets_n<R>(k, g.nz, g.nx * g.ny, o[2]);
        for (int b = 0; b < nb; ++b) {
            double acc = 0.0;
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const double* a = f + (3 * b + ax) * g.S + q;
                double d = s.a[0] * (a[o[ax][0]] - a[o[ax][R]]);
#pragma unroll
                for (int e = 1; e < R; ++e) d += s.a[e] * (a[o[ax][e]] - a[o[ax][R + e]]);
                acc += d;
            }
            div[b * g.S + q] = acc;
        }
    }
}

template <int R>
cudaError_t launch_div(const Grid& g, double dx, const double* f, int nb, double* div, cudaStream_t st) {
    k_divergence<R><<<1216, 256, 0, st>>>(g, make_stencil_n<double, R>(dx), f, nb, div);
    return cudaGetLastError();
}

cudaError_t divergence(const Grid& g, int order, double dx, const double* f, int nb, double* div, cudaStream_t st) {
    switch (stencil_radius(order)) {
        case 1: return launch_div<1>(g, dx, f, nb, div, st);
        case 4: return launch_div<4>(g, dx, f, nb, div, st);
        case 5: return launch_div<5>(g, dx, f, nb, div, st);
        case 6: return launch_div<6>(g, dx, f, nb, div, st);
        default: return launch_div<3>(g, dx, f, nb, div, st);
    }
}

}  // namespace

int ewpt_gauss_project_fp64(const Grid& g, const ewpt_params& p, double* y, int iters, cudaStream_t st,
                            std::string* err);

// Fill an FP64 [36][S] state with the thermal IC (device pointers, stream st).
// gauss_iters < 0: momenta zero (the reference); >= 0: thermal momenta as
// well (amplitude sqrt(n w / V), Higgs streams 4-7, gauge 24 + 4 c), then
// that many iterations of the Gauss projection (gauss.cu).
int ewpt_thermal_fill(const Grid& g, const ewpt_params& p, double T, double mH, double mW, uint64_t seed,
                      double* y, cudaStream_t st, std::string* err, int gauss_iters) {
    const double vol = (double)g.S * p.dx * p.dx * p.dx;
    cufftHandle plan;
    if (cufftPlan3d(&plan, g.nz, g.ny, g.nx, CUFFT_Z2Z) != CUFFT_SUCCESS) {
        *err = "cufftPlan3d (Z2Z) failed";
        return EWPT_ERR_CUFFT;
    }
    cufftSetStream(plan, st);
    cufftDoubleComplex* z = nullptr;
    cudaError_t e = cudaMemsetAsync(y, 0, (size_t)36 * g.S * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&z, (size_t)3 * g.S * sizeof(cufftDoubleComplex), st);
    const uint64_t key = splitmix64(seed);
    const int nb = 1216, nt = 256;
    bool fft_ok = true;
    // y[target] = real(bfft(zc)) (unnormalised backward transform, in place)
    auto to_real = [&](cufftDoubleComplex* zc, int target) {
        if (e != cudaSuccess || !fft_ok) return;
        fft_ok = cufftExecZ2Z(plan, zc, zc, CUFFT_INVERSE) == CUFFT_SUCCESS;
        if (fft_ok) k_real_part<<<nb, nt, 0, st>>>(g.S, zc, y + (size_t)target * g.S);
        e = cudaGetLastError();
    };
    // Higgs phi_1..4: streams 0..3
    const bool mom = gauss_iters >= 0;
    for (int a = 0; a < 4 && e == cudaSuccess; ++a) {
        k_modes_scalar<<<nb, nt, 0, st>>>(g, p.dx, T, mH, vol, key, a, z, 0);
        e = cudaGetLastError();
        to_real(z, a);
        if (mom && e == cudaSuccess && fft_ok) {
            k_modes_scalar<<<nb, nt, 0, st>>>(g, p.dx, T, mH, vol, key, 4 + a, z, 1);
            e = cudaGetLastError();
            to_real(z, 20 + a);
        }
    }
    // W^a (arrays 4 + 3a + i), streams 8 + 4a .. ; Y (13 + i), streams 20 ..;
    // their momenta (24 + 3a + i, 33 + i) streams 24 + 4 c
    for (int c = 0; c < 4 && e == cudaSuccess && fft_ok; ++c) {
        const bool is_y = c == 3;
        k_modes_transverse<<<nb, nt, 0, st>>>(g, p.dx, T, is_y ? 0.0 : mW, vol, key, 8 + 4 * c, z, z + g.S,
                                              z + 2 * g.S, 0);
        e = cudaGetLastError();
        const int base = is_y ? 13 : 4 + 3 * c;
        for (int i = 0; i < 3; ++i) to_real(z + (size_t)i * g.S, base + i);
        if (mom && e == cudaSuccess && fft_ok) {
            k_modes_transverse<<<nb, nt, 0, st>>>(g, p.dx, T, is_y ? 0.0 : mW, vol, key, 24 + 4 * c, z, z + g.S,
                                                  z + 2 * g.S, 1);
            e = cudaGetLastError();
            for (int i = 0; i < 3; ++i) to_real(z + (size_t)i * g.S, 20 + base + i);
        }
    }
    // Gamma^a = div W^a (arrays 16..18), Sigma = div Y (19)
    if (e == cudaSuccess && fft_ok) e = divergence(g, p.stencil_order, p.dx, y + (size_t)4 * g.S, 3, y + (size_t)16 * g.S, st);
    if (e == cudaSuccess && fft_ok) e = divergence(g, p.stencil_order, p.dx, y + (size_t)13 * g.S, 1, y + (size_t)19 * g.S, st);
    if (z) {
        const cudaError_t ef = cudaFreeAsync(z, st);
        if (e == cudaSuccess) e = ef;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cufftDestroy(plan);
    if (!fft_ok) {
        *err = "cufftExecZ2Z failed";
        return EWPT_ERR_CUFFT;
    }
    if (e != cudaSuccess) {
        *err = cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? EWPT_ERR_OOM : EWPT_ERR_CUDA;
    }
    if (gauss_iters > 0) return ewpt_gauss_project_fp64(g, p, y, gauss_iters, st, err);
    return EWPT_OK;
}

int ewpt_check_thermal(double T, double mH, double mW) {
    if (!(std::isfinite(T) && T > 0.0)) return ewpt_fail(nullptr, EWPT_ERR_ARG, "thermal IC: T must be > 0");
    if (!(std::isfinite(mH) && mH >= 0.0 && std::isfinite(mW) && mW >= 0.0))
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "thermal IC: masses must be finite and >= 0");
    return EWPT_OK;
}

extern "C" int ewpt_init_thermal(ewpt_ctx* c, double T, double mH, double mW, uint64_t seed) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    int rc = ewpt_check_thermal(T, mH, mW);
    if (rc) return ewpt_fail(c, rc, "%s", ewpt_last_error(nullptr));
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    cudaSetDevice(c->p.device);
    double* dst;
    rc = ewpt_staging64(c, &dst, true);
    if (rc) return rc;
    std::string err;
    rc = ewpt_thermal_fill(c->g, c->p, T, mH, mW, seed, dst, c->st, &err, -1);
    if (rc) return ewpt_fail(c, rc, "init_thermal: %s", err.c_str());
    cudaError_t e = ewpt_commit_staged(c, dst);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(c, e, "init_thermal");
    if (rc) return rc;
    c->it = 0;
    return EWPT_OK;
}

// Thermal IC from the caller's deviate arrays (the reference's construction,
// main_rk4.jl:5348-5636, with its random draws supplied): dev holds 44
// arrays of S doubles, host or device memory -- for W^1, W^2, W^3 and Y the
// ten arrays r_1, r_2, r_3, r_1_i, r_2_i, r_3_i, x_1, x_2, x_3, x_4 in the
// order run() draws them, then phi_1_k .. phi_4_k.  Gamma, Sigma and the
// momenta are zero, as in run().
extern "C" int ewpt_init_thermal_deviates(ewpt_ctx* c, double T, double mH, double mW, const double* dev,
                                          int32_t on_device, int32_t flags) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!dev) return ewpt_fail(c, EWPT_ERR_ARG, "deviates is NULL");
    if (flags & ~EWPT_THERMAL_ONE_BASED_MODES) return ewpt_fail(c, EWPT_ERR_ARG, "unknown thermal flags %d", flags);
    int rc = ewpt_check_thermal(T, mH, mW);
    if (rc) return ewpt_fail(c, rc, "%s", ewpt_last_error(nullptr));
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    cudaSetDevice(c->p.device);
    double* y;
    rc = ewpt_staging64(c, &y, true);
    if (rc) return rc;
    const Grid& g = c->g;
    const cudaStream_t st = c->st;
    const double vol = (double)g.S * c->p.dx * c->p.dx * c->p.dx;
    const int one_based = (flags & EWPT_THERMAL_ONE_BASED_MODES) ? 1 : 0;
    cufftHandle plan;
    if (cufftPlan3d(&plan, g.nz, g.ny, g.nx, CUFFT_Z2Z) != CUFFT_SUCCESS)
        return ewpt_fail(c, EWPT_ERR_CUFFT, "cufftPlan3d (Z2Z) failed");
    cufftSetStream(plan, st);
    cufftDoubleComplex* z = nullptr;
    double* d = nullptr;  // device copy of one group's deviates (host input)
    cudaError_t e = cudaMemsetAsync(y, 0, (size_t)36 * g.S * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&z, (size_t)3 * g.S * sizeof(cufftDoubleComplex), st);
    if (e == cudaSuccess && !on_device) e = cudaMallocAsync(&d, (size_t)10 * g.S * 8, st);
    bool fft_ok = true;
    const int nb = 1216, nt = 256;
    auto group = [&](int first, int n) -> const double* {
        const double* src = dev + (size_t)first * g.S;
        if (on_device || e != cudaSuccess) return src;
        e = cudaMemcpyAsync(d, src, (size_t)n * g.S * 8, cudaMemcpyHostToDevice, st);
        return d;
    };
    auto to_real = [&](cufftDoubleComplex* zc, int target) {
        if (e != cudaSuccess || !fft_ok) return;
        fft_ok = cufftExecZ2Z(plan, zc, zc, CUFFT_INVERSE) == CUFFT_SUCCESS;
        if (fft_ok) k_real_part<<<nb, nt, 0, st>>>(g.S, zc, y + (size_t)target * g.S);
        e = cudaGetLastError();
    };
    for (int gi = 0; gi < 4 && e == cudaSuccess && fft_ok; ++gi) {
        const double* dd = group(10 * gi, 10);
        if (e != cudaSuccess) break;
        k_dev_transverse<<<nb, nt, 0, st>>>(g, c->p.dx, T, gi == 3 ? 0.0 : mW, vol, one_based, dd, z, z + g.S,
                                            z + 2 * g.S);
        e = cudaGetLastError();
        const int base = gi == 3 ? 13 : 4 + 3 * gi;
        for (int i = 0; i < 3; ++i) to_real(z + (size_t)i * g.S, base + i);
    }
    for (int a = 0; a < 4 && e == cudaSuccess && fft_ok; ++a) {
        const double* dd = group(40 + a, 1);
        if (e != cudaSuccess) break;
        k_dev_scalar<<<nb, nt, 0, st>>>(g, c->p.dx, T, mH, vol, one_based, dd, z);
        e = cudaGetLastError();
        to_real(z, a);
    }
    if (z) {
        const cudaError_t ef = cudaFreeAsync(z, st);
        if (e == cudaSuccess) e = ef;
    }
    if (d) {
        const cudaError_t ef = cudaFreeAsync(d, st);
        if (e == cudaSuccess) e = ef;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cufftDestroy(plan);
    if (!fft_ok) return ewpt_fail(c, EWPT_ERR_CUFFT, "cufftExecZ2Z failed");
    rc = ewpt_cuda_check(c, e, "init_thermal_deviates");
    if (rc) return rc;
    e = ewpt_commit_staged(c, y);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rc = ewpt_cuda_check(c, e, "init_thermal_deviates");
    if (rc) return rc;
    c->it = 0;
    return EWPT_OK;
}

// The thermal IC with thermal momenta projected onto the Gauss law (the
// benchmark's precision configuration: "momenta set by the Gauss-constraint
// projection"); gauss_iters iterations of gauss.cu's projection.
extern "C" int ewpt_init_thermal_gauss(ewpt_ctx* c, double T, double mH, double mW, uint64_t seed,
                                       int32_t gauss_iters) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    int rc = ewpt_check_thermal(T, mH, mW);
    if (rc) return ewpt_fail(c, rc, "%s", ewpt_last_error(nullptr));
    if (gauss_iters < 0) return ewpt_fail(c, EWPT_ERR_ARG, "gauss_iters < 0");
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    if (c->p.stencil_order != 6) return ewpt_fail(c, EWPT_ERR_ARG, "the projection uses the 6th-order stencil");
    cudaSetDevice(c->p.device);
    double* dst;
    rc = ewpt_staging64(c, &dst, true);
    if (rc) return rc;
    std::string err;
    rc = ewpt_thermal_fill(c->g, c->p, T, mH, mW, seed, dst, c->st, &err, gauss_iters);
    if (rc) return ewpt_fail(c, rc, "init_thermal_gauss: %s", err.c_str());
    cudaError_t e = ewpt_commit_staged(c, dst);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(c, e, "init_thermal_gauss");
    if (rc) return rc;
    c->it = 0;
    return EWPT_OK;
}
