// init.cu -- bubble-nucleation initial conditions on the device.
//
// Reference: initializer! adds one bubble's profile to phi per launch
// (gpu-kernels-rk4/main_rk4.jl:4930-4946, called once per bubble at
// :5691-5697).  Here one kernel sums every bubble of a list at each site, in
// FP64, and writes the whole state (phi = sum of profiles, everything else
// zero) of a single lattice (FP64 or FP32 form) or of an ensemble member.
//
// profile 0 (reference): rmag(rb) of initializer!, with the reference's
//   sin-distance rb = sqrt(sum_i sin^2(rk_i ((x_i - 1) - (c_i - 0.5)) dx)/rk_i^2),
//   rk_i = pi/((n_i - 1) dx), centres c in the reference's 1-based indices.
// profile 1 (benchmark configurations): 0.5 vev (1 - tanh((r - R)/w)) with r
//   the minimum-image distance to the centre (physical units) -- the same
//   formula as ewpt/ic.py bubbles_tanh.
#include <cmath>
#include <vector>

#include "ewpt_ctx.cuh"

namespace {

struct Bubble {
    double cx, cy, cz;
    double d1, d2, d3, d4;
};

__device__ __forceinline__ double min_image(double d, double L) { return d - L * rint(d / L); }

// Writes phi (arrays 0..3) and zeros the other 32 arrays of one [36][S] state.
template <typename Out>
__global__ void k_bubbles(int nx, int ny, int nz, double dx, const Bubble* __restrict__ bub, int nb, int profile,
                          double p0, double p1, double p2, Out out) {
    const int64_t S = (int64_t)nx * ny * nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < S; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const int j = (int)((c / nx) % ny);
        const int k = (int)(c / ((int64_t)nx * ny));
        double f1 = 0, f2 = 0, f3 = 0, f4 = 0;
        for (int b = 0; b < nb; ++b) {
            const Bubble B = bub[b];
            double prof;
            if (profile == 0) {
                // p0 = mH; rk_i = pi/((n_i - 1) dx)
                const double rkx = M_PI / ((nx - 1) * dx), rky = M_PI / ((ny - 1) * dx), rkz = M_PI / ((nz - 1) * dx);
                const double sx = sin(rkx * (i - (B.cx - 0.5)) * dx);
                const double sy = sin(rky * (j - (B.cy - 0.5)) * dx);
                const double sz = sin(rkz * (k - (B.cz - 0.5)) * dx);
                const double rb = sqrt(sx * sx / (rkx * rkx) + sy * sy / (rky * rky) + sz * sz / (rkz * rkz));
                const double s2 = sqrt(2.0), q = (s2 - 1.0) * (s2 - 1.0);
                prof = (1.0 + q) * exp(-p0 * rb / s2) / (1.0 + q * exp(-s2 * p0 * rb));
            } else {
                // p0 = R, p1 = w, p2 = vev
                const double ddx = min_image(i * dx - B.cx, nx * dx);
                const double ddy = min_image(j * dx - B.cy, ny * dx);
                const double ddz = min_image(k * dx - B.cz, nz * dx);
                const double r = sqrt(ddz * ddz + ddy * ddy + ddx * ddx);
                prof = p2 * 0.5 * (1.0 - tanh((r - p0) / p1));
            }
            f1 += B.d1 * prof;
            f2 += B.d2 * prof;
            f3 += B.d3 * prof;
            f4 += B.d4 * prof;
        }
        out(0, c, f1);
        out(1, c, f2);
        out(2, c, f3);
        out(3, c, f4);
        for (int a = 4; a < 36; ++a) out(a, c, 0.0);
    }
}

struct OutF64 {
    double* y;
    int64_t S;
    __device__ void operator()(int a, int64_t c, double v) const { y[a * S + c] = v; }
};
struct OutHiLo {
    float* hi;
    float* lo;
    Grid g;
    Layout L;
    __device__ void operator()(int a, int64_t c, double v) const {
        const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((int64_t)g.nx * g.ny));
        const int64_t q = a * L.P + L.at(i, j, k);
        const float h = (float)v;
        hi[q] = h;
        lo[q] = (float)(v - (double)h);
    }
};

}  // namespace

// Launch the bubble kernel on a state given as FP64 [36][S] (y != null) or
// as FP32 hi/lo [36][S] pairs.  bubbles: nb x 7 doubles (centre, direction).
int ewpt_launch_bubbles(const Grid& g, double dx, int nb, const double* bubbles, int profile, double p0, double p1,
                        double p2, double* y, float* hi, float* lo, const Layout& L, cudaStream_t st,
                        std::string* err) {
    Bubble* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, sizeof(Bubble) * (nb > 0 ? nb : 1), st);
    if (e == cudaSuccess && nb > 0) e = cudaMemcpyAsync(d, bubbles, sizeof(Bubble) * nb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        if (y)
            k_bubbles<<<1216, 256, 0, st>>>(g.nx, g.ny, g.nz, dx, d, nb, profile, p0, p1, p2, OutF64{y, g.S});
        else
            k_bubbles<<<1216, 256, 0, st>>>(g.nx, g.ny, g.nz, dx, d, nb, profile, p0, p1, p2, OutHiLo{hi, lo, g, L});
        e = cudaGetLastError();
        if (e == cudaSuccess && !y) e = launch_ghost_fill(g, L, hi, st, true);
    }
    if (d) cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess && err) *err = cudaGetErrorString(e);
    return e == cudaSuccess ? EWPT_OK : EWPT_ERR_CUDA;
}

static int check_bubbles(int32_t nb, const double* bubbles, int32_t profile, double p0, double p1) {
    if (nb < 0 || (nb > 0 && !bubbles)) return ewpt_fail(nullptr, EWPT_ERR_ARG, "bubble list");
    if (profile != EWPT_BUBBLE_REFERENCE && profile != EWPT_BUBBLE_TANH)
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "profile %d unknown", profile);
    for (int64_t q = 0; q < 7 * (int64_t)nb; ++q)
        if (!std::isfinite(bubbles[q])) return ewpt_fail(nullptr, EWPT_ERR_ARG, "non-finite bubble entry");
    if (!std::isfinite(p0) || !std::isfinite(p1) || (profile == EWPT_BUBBLE_TANH && !(p1 > 0)))
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "bad profile parameters");
    return EWPT_OK;
}

extern "C" int ewpt_init_bubbles(ewpt_ctx* c, int32_t nb, const double* bubbles, int32_t profile, double p0,
                                 double p1) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    int rc = check_bubbles(nb, bubbles, profile, p0, p1);
    if (rc) return ewpt_fail(c, rc, "%s", ewpt_last_error(nullptr));
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    cudaSetDevice(c->p.device);
    const double q0 = profile == EWPT_BUBBLE_REFERENCE ? c->p.mH : p0;
    std::string err;
    rc = c->p.precision != EWPT_FP32
             ? ewpt_launch_bubbles(c->g, c->p.dx, nb, bubbles, profile, q0, p1, c->p.vev, c->y, nullptr, nullptr,
                                   c->lay, c->st, &err)
             : ewpt_launch_bubbles(c->g, c->p.dx, nb, bubbles, profile, q0, p1, c->p.vev, nullptr, c->y32.hi,
                                   c->y32.lo, c->lay, c->st, &err);
    if (rc) return ewpt_fail(c, rc, "init_bubbles: %s", err.c_str());
    if (c->p.precision == EWPT_DF64) {
        rc = ewpt_cuda_check(c, launch_to_dd(36 * c->g.S, c->y, c->st), "init_bubbles");
        if (rc) return rc;
    }
    c->it = 0;
    return EWPT_OK;
}
