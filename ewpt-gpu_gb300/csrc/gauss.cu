// gauss.cu -- projection of an FP64 state's electric fields onto the
// discrete Gauss law, on the device.
//
// The Gauss constraints of the evolution are the gp2 parts of k_Gamma and
// k_Sigma (main_rk4.jl:603-655): d_i E^a_i = rho^a with
//   rho^a = g (Higgs charge  phi^T M_a pi  -  sum_i (W^b_i E^c_i - W^c_i E^b_i))
// for (a, b, c) cyclic, and d_i E^Y_i = rho_Y = g' phi^T M_Y pi, where E are
// the gauge momenta, pi the Higgs momenta and d_i the 6th-order central
// difference.  A thermal state draws E and pi freely; one projection
// iteration makes it satisfy the constraints:
//   1. neutralise: the central-difference divergence cannot produce the zero
//      mode or the staggered modes (-1)^(e.x) (e_i = 1 only on even axes), so
//      the charges must have no component there.  The Higgs momenta move
//      along the charge generators, pi += sum_b c_b(x) M_b^T phi with c_b
//      constant on each of the 8 parity classes of the sites; the 4 x ne
//      coefficients solve a least-squares system whose entries are
//      parity-class moments of rho and of phi^T M_a M_b^T phi (one reduction
//      kernel, then a one-sided Jacobi SVD of the <= 32 x 32 system on the
//      host, the minimum-norm solution as numpy's lstsq gives it);
//   2. project: per group (the three SU(2) colours and U(1)), with rho taken
//      before the iteration, E <- E - grad chi with d.d chi = d.E - rho solved
//      in Fourier space with the derivative's symbol
//      s(theta) = (90 sin theta - 18 sin 2 theta + 2 sin 3 theta) / (60 dx)
//      (cuFFT D2Z / Z2D); modes with |s|^2 <= 1e-12 max |s|^2 are left alone.
// The rho^a of the next iteration sees the projected E (the SU(2) charge
// depends on E), so the residual falls by iterations.  This is the device
// version of ewpt/ic.py gauss_project (same steps, same order).
#include <cufft.h>

#include <cmath>
#include <string>
#include <vector>

#include "ewpt_ctx.cuh"

namespace {

constexpr int kNQ = 20;  // moments per parity class: 4 charges, then 16 generator overlaps

// charge generators M_a (a = 0, 1, 2: SU(2); 3: U(1)): M[i][j] = 1, M[j][i] = -1 per pair
__constant__ int kPairs[4][2][2] = {{{0, 3}, {2, 1}}, {{2, 0}, {3, 1}}, {{0, 1}, {3, 2}}, {{0, 1}, {2, 3}}};

// u = M_b^T phi
__device__ __forceinline__ void gen_t(int b, const double* ph, double* u) {
    u[0] = u[1] = u[2] = u[3] = 0.0;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = kPairs[b][q][0], j = kPairs[b][q][1];
        u[j] += ph[i];
        u[i] -= ph[j];
    }
}

// rho^1..3 and rho_Y at site c of an FP64 [36][S] state
__device__ __forceinline__ void site_charges(const double* __restrict__ y, int64_t S, int64_t c, double gw, double gy,
                                             double* rho) {
    double ph[4], pi[4], u[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ph[a] = y[a * S + c];
        pi[a] = y[(20 + a) * S + c];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        gen_t(a, ph, u);  // phi^T M_a pi = (M_a^T phi) . pi
        double h = u[0] * pi[0] + u[1] * pi[1] + u[2] * pi[2] + u[3] * pi[3];
        if (a < 3) {
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            double q = 0.0;
#pragma unroll
            for (int i = 0; i < 3; ++i)
                q -= y[(4 + 3 * b + i) * S + c] * y[(24 + 3 * cc + i) * S + c] -
                     y[(4 + 3 * cc + i) * S + c] * y[(24 + 3 * b + i) * S + c];
            rho[a] = gw * q + gw * h;
        } else {
            rho[a] = gy * h;
        }
    }
}

__global__ void k_charges(Grid g, const double* __restrict__ y, double gw, double gy, double* __restrict__ rho) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        double r[4];
        site_charges(y, g.S, q, gw, gy, r);
#pragma unroll
        for (int a = 0; a < 4; ++a) rho[a * g.S + q] = r[a];
    }
}

__device__ __forceinline__ int parity_class(const Grid& g, int64_t q) {
    const int i = (int)(q % g.nx), j = (int)((q / g.nx) % g.ny), k = (int)(q / ((int64_t)g.nx * g.ny));
    return (k & 1) * 4 + (j & 1) * 2 + (i & 1);
}

// per-block sums over each parity class of the 4 charges and of the 16
// coup_a (M_a^T phi).(M_b^T phi); part[block][class][kNQ]
__global__ void __launch_bounds__(256) k_class_moments(Grid g, const double* __restrict__ y, double gw, double gy,
                                                       double* __restrict__ part) {
    __shared__ double sh[8 * kNQ];
    for (int t = threadIdx.x; t < 8 * kNQ; t += blockDim.x) sh[t] = 0.0;
    __syncthreads();
    const double coup[4] = {gw, gw, gw, gy};
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        double v[kNQ], ph[4], u[4][4];
        site_charges(y, g.S, q, gw, gy, v);
#pragma unroll
        for (int a = 0; a < 4; ++a) ph[a] = y[a * g.S + q];
#pragma unroll
        for (int b = 0; b < 4; ++b) gen_t(b, ph, u[b]);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
                v[4 + 4 * a + b] =
                    coup[a] * (u[a][0] * u[b][0] + u[a][1] * u[b][1] + u[a][2] * u[b][2] + u[a][3] * u[b][3]);
        double* s = sh + parity_class(g, q) * kNQ;
#pragma unroll
        for (int t = 0; t < kNQ; ++t) atomicAdd(s + t, v[t]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 8 * kNQ; t += blockDim.x) part[(int64_t)blockIdx.x * 8 * kNQ + t] = sh[t];
}

// pi += table[b][class(x)] M_b^T phi
__global__ void k_shift_momenta(Grid g, double* __restrict__ y, const double* __restrict__ table) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < g.S; q += (int64_t)gridDim.x * blockDim.x) {
        const int cls = parity_class(g, q);
        double ph[4], u[4], d[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int a = 0; a < 4; ++a) ph[a] = y[a * g.S + q];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            gen_t(b, ph, u);
            const double t = table[b * 8 + cls];
#pragma unroll
            for (int a = 0; a < 4; ++a) d[a] += t * u[a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) y[(20 + a) * g.S + q] += d[a];
    }
}

__device__ __forceinline__ double deriv_symbol(double th, double dx) {
    return (90.0 * sin(th) - 18.0 * sin(2.0 * th) + 2.0 * sin(3.0 * th)) / (60.0 * dx);
}

// half spectrum (x: 0..nx/2): C0..C2 = FFT(E_x, E_y, E_z), C3 = FFT(rho);
// C_j <- (C_j - i s_j chi) / S, chi = (i s.C - C3) / (-|s|^2) where |s|^2 > cut
__global__ void k_project_modes(Grid g, double dx, double cut, cufftDoubleComplex* __restrict__ c0,
                                cufftDoubleComplex* __restrict__ c1, cufftDoubleComplex* __restrict__ c2,
                                const cufftDoubleComplex* __restrict__ c3) {
    const int hx = g.nx / 2 + 1;
    const int64_t H = (int64_t)hx * g.ny * g.nz;
    const double inv = 1.0 / (double)g.S, two_pi = 6.283185307179586;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < H; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % hx), j = (int)((q / hx) % g.ny), k = (int)(q / ((int64_t)hx * g.ny));
        const double sx = deriv_symbol(two_pi * i / g.nx, dx), sy = deriv_symbol(two_pi * j / g.ny, dx),
                     sz = deriv_symbol(two_pi * k / g.nz, dx);
        const double s2 = sx * sx + sy * sy + sz * sz;
        const cufftDoubleComplex a = c0[q], b = c1[q], c = c2[q], r = c3[q];
        double chr = 0.0, chi = 0.0;
        if (s2 > cut) {
            // res = i (s . C) - rho_hat
            const double re = -(sx * a.y + sy * b.y + sz * c.y) - r.x;
            const double im = (sx * a.x + sy * b.x + sz * c.x) - r.y;
            chr = -re / s2;
            chi = -im / s2;
        }
        // C_j - i s_j chi: (x + i y) - i s (u + i v) = (x + s v) + i (y - s u)
        c0[q] = make_cuDoubleComplex((a.x + sx * chi) * inv, (a.y - sx * chr) * inv);
        c1[q] = make_cuDoubleComplex((b.x + sy * chi) * inv, (b.y - sy * chr) * inv);
        c2[q] = make_cuDoubleComplex((c.x + sz * chi) * inv, (c.y - sz * chr) * inv);
    }
}

double host_symbol(double th, double dx) {
    return (90.0 * std::sin(th) - 18.0 * std::sin(2.0 * th) + 2.0 * std::sin(3.0 * th)) / (60.0 * dx);
}

// The staggered vectors e = (ez, ey, ex), e_i = 1 only on even axes, ez outermost.
std::vector<int> null_vectors(const Grid& g) {
    std::vector<int> es;
    for (int ez = 0; ez < (g.nz % 2 == 0 ? 2 : 1); ++ez)
        for (int ey = 0; ey < (g.ny % 2 == 0 ? 2 : 1); ++ey)
            for (int ex = 0; ex < (g.nx % 2 == 0 ? 2 : 1); ++ex) es.push_back(ez * 4 + ey * 2 + ex);
    return es;
}

// sum_x (-1)^(e.x) f(x) from the parity-class sums s[class] (class = pz*4 + py*2 + px)
double moment(const double* s, int stride, int e) {
    double m = 0.0;
    for (int c = 0; c < 8; ++c) m += (__builtin_popcount(c & e) & 1 ? -1.0 : 1.0) * s[c * stride];
    return m;
}

// Minimum-norm least-squares solution of A x = b (m x n, row-major), by a
// one-sided Jacobi SVD (Hestenes); singular values below
// eps * max(m, n) * sigma_max are dropped, as numpy's lstsq does by default.
std::vector<double> lstsq(std::vector<double> A, int m, int n, const std::vector<double>& b) {
    std::vector<double> V((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int i = 0; i < m; ++i) {
                    const double x = A[(size_t)i * n + p], y = A[(size_t)i * n + q];
                    al += x * x;
                    be += y * y;
                    ga += x * y;
                }
                if (ga == 0.0 || std::fabs(ga) <= 1e-15 * std::sqrt(al * be)) continue;
                off = std::fmax(off, std::fabs(ga) / std::sqrt(al * be));
                const double zeta = (be - al) / (2.0 * ga);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < m; ++i) {
                    const double x = A[(size_t)i * n + p], y = A[(size_t)i * n + q];
                    A[(size_t)i * n + p] = c * x - s * y;
                    A[(size_t)i * n + q] = s * x + c * y;
                }
                for (int i = 0; i < n; ++i) {
                    const double x = V[(size_t)i * n + p], y = V[(size_t)i * n + q];
                    V[(size_t)i * n + p] = c * x - s * y;
                    V[(size_t)i * n + q] = s * x + c * y;
                }
            }
        if (off < 1e-15) break;
    }
    std::vector<double> sig(n), x(n, 0.0);
    double smax = 0.0;
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int i = 0; i < m; ++i) s += A[(size_t)i * n + k] * A[(size_t)i * n + k];
        sig[k] = std::sqrt(s);
        smax = std::fmax(smax, sig[k]);
    }
    const double tol = 2.220446049250313e-16 * (m > n ? m : n) * smax;
    for (int k = 0; k < n; ++k) {
        if (!(sig[k] > tol)) continue;
        double ub = 0.0;  // u_k . b, u_k = A[:, k] / sigma_k
        for (int i = 0; i < m; ++i) ub += A[(size_t)i * n + k] * b[i];
        const double w = ub / (sig[k] * sig[k]);
        for (int j = 0; j < n; ++j) x[j] += V[(size_t)j * n + k] * w;
    }
    return x;
}

}  // namespace

// Project the electric fields (and neutralise the charges through the Higgs
// momenta) of an FP64 [36][S] device state in place: `iters` iterations.
int ewpt_gauss_project_fp64(const Grid& g, const ewpt_params& p, double* y, int iters, cudaStream_t st,
                            std::string* err) {
    if (iters <= 0) return EWPT_OK;
    const int nb = 1216, nt = 256;
    const int hx = g.nx / 2 + 1;
    const int64_t H = (int64_t)hx * g.ny * g.nz;
    cufftHandle fwd = 0, inv = 0;
    if (cufftPlan3d(&fwd, g.nz, g.ny, g.nx, CUFFT_D2Z) != CUFFT_SUCCESS ||
        cufftPlan3d(&inv, g.nz, g.ny, g.nx, CUFFT_Z2D) != CUFFT_SUCCESS) {
        if (fwd) cufftDestroy(fwd);
        *err = "cufftPlan3d (D2Z/Z2D) failed";
        return EWPT_ERR_CUFFT;
    }
    cufftSetStream(fwd, st);
    cufftSetStream(inv, st);
    double *rho = nullptr, *part = nullptr, *table = nullptr;
    cufftDoubleComplex* C = nullptr;
    cudaError_t e = cudaMallocAsync(&rho, (size_t)4 * g.S * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&C, (size_t)4 * H * sizeof(cufftDoubleComplex), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&part, (size_t)nb * 8 * kNQ * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&table, 32 * 8, st);
    // |s|^2 cut: 1e-12 of its largest value (the sum of each axis' largest)
    double smax = 0.0;
    const int N[3] = {g.nx, g.ny, g.nz};
    for (int d = 0; d < 3; ++d) {
        double m = 0.0;
        for (int n = 0; n < N[d]; ++n) m = std::fmax(m, std::pow(host_symbol(6.283185307179586 * n / N[d], p.dx), 2));
        smax += m;
    }
    const double cut = 1e-12 * smax;
    const std::vector<int> es = null_vectors(g);
    const int ne = (int)es.size(), n = 4 * ne;
    std::vector<double> hp((size_t)nb * 8 * kNQ), sums(8 * kNQ);
    bool fft_ok = true;
    for (int it = 0; it < iters && e == cudaSuccess && fft_ok; ++it) {
        // 1. neutralise the charges' null-mode components
        k_class_moments<<<nb, nt, 0, st>>>(g, y, p.gw, p.gy, part);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, hp.size() * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        std::fill(sums.begin(), sums.end(), 0.0);
        for (int b = 0; b < nb; ++b)
            for (int t = 0; t < 8 * kNQ; ++t) sums[t] += hp[(size_t)b * 8 * kNQ + t];
        std::vector<double> A((size_t)n * n), Q(n);
        for (int a = 0; a < 4; ++a) {
            for (int i = 0; i < ne; ++i) Q[a * ne + i] = -moment(&sums[a], kNQ, es[i]);
            for (int b = 0; b < 4; ++b)
                for (int i = 0; i < ne; ++i)
                    for (int j = 0; j < ne; ++j)
                        A[(size_t)(a * ne + i) * n + b * ne + j] = moment(&sums[4 + 4 * a + b], kNQ, es[i] ^ es[j]);
        }
        const std::vector<double> alpha = lstsq(A, n, n, Q);
        double tab[32];
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 8; ++c) {
                double t = 0.0;
                for (int j = 0; j < ne; ++j) t += alpha[b * ne + j] * (__builtin_popcount(c & es[j]) & 1 ? -1.0 : 1.0);
                tab[b * 8 + c] = t;
            }
        e = cudaMemcpyAsync(table, tab, sizeof tab, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) k_shift_momenta<<<nb, nt, 0, st>>>(g, y, table);
        // 2. charges of this iteration, then each group's projection
        if (e == cudaSuccess) k_charges<<<nb, nt, 0, st>>>(g, y, p.gw, p.gy, rho);
        if (e == cudaSuccess) e = cudaGetLastError();
        for (int grp = 0; grp < 4 && e == cudaSuccess && fft_ok; ++grp) {
            double* E = y + (size_t)(grp < 3 ? 24 + 3 * grp : 33) * g.S;
            for (int i = 0; i < 3 && fft_ok; ++i) fft_ok = cufftExecD2Z(fwd, E + (size_t)i * g.S, C + i * H) == CUFFT_SUCCESS;
            if (fft_ok) fft_ok = cufftExecD2Z(fwd, rho + (size_t)grp * g.S, C + 3 * H) == CUFFT_SUCCESS;
            if (!fft_ok) break;
            k_project_modes<<<nb, nt, 0, st>>>(g, p.dx, cut, C, C + H, C + 2 * H, C + 3 * H);
            e = cudaGetLastError();
            for (int i = 0; i < 3 && fft_ok && e == cudaSuccess; ++i)
                fft_ok = cufftExecZ2D(inv, C + i * H, E + (size_t)i * g.S) == CUFFT_SUCCESS;
        }
    }
    const cudaError_t ef[4] = {rho ? cudaFreeAsync(rho, st) : cudaSuccess, C ? cudaFreeAsync(C, st) : cudaSuccess,
                               part ? cudaFreeAsync(part, st) : cudaSuccess, table ? cudaFreeAsync(table, st) : cudaSuccess};
    for (cudaError_t x : ef)
        if (e == cudaSuccess) e = x;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cufftDestroy(fwd);
    cufftDestroy(inv);
    if (!fft_ok) {
        *err = "cuFFT execution failed";
        return EWPT_ERR_CUFFT;
    }
    if (e != cudaSuccess) {
        *err = cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? EWPT_ERR_OOM : EWPT_ERR_CUDA;
    }
    return EWPT_OK;
}

extern "C" int ewpt_gauss_project(ewpt_ctx* c, int32_t iters) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (iters < 0) return ewpt_fail(c, EWPT_ERR_ARG, "iterations < 0");
    if (c->view || c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "needs a whole-lattice context");
    if (c->p.stencil_order != 6) return ewpt_fail(c, EWPT_ERR_ARG, "the projection uses the 6th-order stencil");
    cudaSetDevice(c->p.device);
    // the FP64 state, or the FP32/DF64 form's state joined into FP64
    const double* cur;
    int rc = ewpt_state64(c, &cur);
    if (rc) return rc;
    double* y = const_cast<double*>(cur);
    std::string err;
    rc = ewpt_gauss_project_fp64(c->g, c->p, y, iters, c->st, &err);
    if (rc) return ewpt_fail(c, rc, "gauss_project: %s", err.c_str());
    cudaError_t e = cudaSuccess;
    if (c->p.precision == EWPT_DF64) {
        // the pairs were joined into scratch64; they are made again in place in c->y
        e = cudaMemcpyAsync(c->y, y, (size_t)36 * c->g.S * 8, cudaMemcpyDeviceToDevice, c->st);
        if (e == cudaSuccess) e = ewpt_commit_staged(c, c->y);
    } else if (c->p.precision == EWPT_FP32) {
        e = ewpt_commit_staged(c, y);  // split into hi/lo with the ghost images
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    return ewpt_cuda_check(c, e, "gauss_project");
}
