// spectrum.cu -- B-field and Higgs power spectra: cuFFT D2Z + shell binning.
//
// Reference: the B components are FFT'd with CUFFT (main_rk4.jl:6580-6685)
// and P = |Bx^|^2 + |By^|^2 + |Bz^|^2 is binned on the host by sorting all N^3
// modes (convolve_1d, spec_routines.jl:47-77; integer lattice |n| from the
// wrapped index, K_c_mag :6-30).  Here the transform is a real-to-complex
// D2Z (half the bytes of the reference's complex transform of a real field)
// and the binning is a device kernel over the half spectrum, each mode
// weighted by its multiplicity in the full spectrum (2, or 1 on the kx = 0
// and kx = nx/2 planes).
//
//   mode EWPT_SPEC_LOG    : nbins log-spaced shells in |n| over [1, nmax],
//                           nmax = min(nx,ny,nz)/2, DC excluded.  Per-block
//                           partial histograms in shared memory, folded in a
//                           fixed order (deterministic).
//   mode EWPT_SPEC_UNIQUE : one bin per distinct integer |n|^2 (the
//                           reference's convolve_1d), first nbins distinct
//                           values in increasing order; FP64 atomics.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ewpt_ctx.cuh"

cudaError_t launch_fields(const Grid& g, const ewpt_params& p, const double* y, int which, double* f,
                          cudaStream_t st);

namespace {

constexpr int MAXSHELL = 256;
constexpr int SB = 256;  // threads per binning block

__device__ __forceinline__ int wrapk(int x, int n) { return x <= n / 2 ? x : x - n; }

// Integer |n|^2 threshold table: mode m belongs to shell b when
// thr[b] <= m < thr[b+1]; thr[nbins] = nmax^2 + 1.
__global__ void k_bin_log(int nx, int ny, int nz, int nxh, const cufftDoubleComplex* __restrict__ F,
                          const int64_t* __restrict__ thr, int nbins, int count_modes, double* __restrict__ part) {
    __shared__ double ssum[MAXSHELL];
    __shared__ double scnt[MAXSHELL];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        ssum[b] = 0.0;
        scnt[b] = 0.0;
    }
    __syncthreads();
    const int64_t nh = (int64_t)nxh * ny * nz;
    const int64_t mmax = thr[nbins] - 1;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nh; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % nxh);
        const int64_t r = q / nxh;
        const int y = (int)(r % ny);
        const int z = (int)(r / ny);
        const int kx = x, ky = wrapk(y, ny), kz = wrapk(z, nz);
        const int64_t m = (int64_t)kx * kx + (int64_t)ky * ky + (int64_t)kz * kz;
        if (m == 0 || m > mmax) continue;
        // binary search the shell
        int lo = 0, hi = nbins;  // thr[lo] <= m < thr[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (thr[mid] <= m) lo = mid; else hi = mid;
        }
        const cufftDoubleComplex f = F[q];
        const double w = (x == 0 || (2 * x == nx)) ? 1.0 : 2.0;
        const double p = (f.x * f.x + f.y * f.y) * w;
        atomicAdd(&ssum[lo], p);
        if (count_modes) atomicAdd(&scnt[lo], w);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        part[(int64_t)blockIdx.x * 2 * nbins + b] += ssum[b];
        part[(int64_t)blockIdx.x * 2 * nbins + nbins + b] += scnt[b];
    }
}

__global__ void k_bin_fold(const double* __restrict__ part, int nblk, int nbins, double* __restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= 2 * nbins) return;
    double v = 0.0;
    for (int k = 0; k < nblk; ++k) v += part[(int64_t)k * 2 * nbins + b];
    out[b] = v;
}

// Unique-|n|^2 histogram (sum and count) over m in [0, mmax].
__global__ void k_bin_unique(int nx, int ny, int nz, int nxh, const cufftDoubleComplex* __restrict__ F,
                             int64_t mmax, int zero_dc, int count_modes, double* __restrict__ hsum,
                             double* __restrict__ hcnt) {
    const int64_t nh = (int64_t)nxh * ny * nz;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nh; q += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % nxh);
        const int64_t r = q / nxh;
        const int y = (int)(r % ny);
        const int z = (int)(r / ny);
        const int kx = x, ky = wrapk(y, ny), kz = wrapk(z, nz);
        const int64_t m = (int64_t)kx * kx + (int64_t)ky * ky + (int64_t)kz * kz;
        if (m > mmax) continue;
        const cufftDoubleComplex f = F[q];
        const double w = (x == 0 || (2 * x == nx)) ? 1.0 : 2.0;
        double p = (f.x * f.x + f.y * f.y) * w;
        if (zero_dc && m == 0) p = 0.0;
        atomicAdd(&hsum[m], p);
        if (count_modes) atomicAdd(&hcnt[m], w);
    }
}

inline int64_t ipow2(int64_t a) { return a * a; }

}  // namespace

// Integer |n|^2 thresholds of nbins log shells over |n| in [1, nmax].
std::vector<int64_t> ewpt_shell_thresholds(int nmax, int nbins) {
    std::vector<int64_t> t(nbins + 1);
    const double lmax = std::log((double)nmax);
    for (int b = 0; b <= nbins; ++b) {
        if (b == 0) {
            t[b] = 1;
            continue;
        }
        if (b == nbins) {
            t[b] = ipow2(nmax) + 1;
            continue;
        }
        const double e = std::exp(lmax * (double)b / (double)nbins);
        int64_t m = (int64_t)std::ceil(e * e);
        while (m > 1 && std::sqrt((double)(m - 1)) >= e) --m;
        while (std::sqrt((double)m) < e) ++m;
        t[b] = m;
    }
    return t;
}

extern "C" {

int64_t ewpt_kc_bin_nums(int32_t cx, int32_t cy, int32_t cz) {
    if (cx < 1 || cy < 1 || cz < 1) return -1;
    std::vector<int64_t> v;
    v.reserve((size_t)cx * cy * cz);
    for (int i = 0; i < cx; ++i)
        for (int j = 0; j < cy; ++j)
            for (int k = 0; k < cz; ++k) {
                const int64_t a = i <= cx / 2 ? i : i - cx, b = j <= cy / 2 ? j : j - cy, c = k <= cz / 2 ? k : k - cz;
                v.push_back(a * a + b * b + c * c);
            }
    std::sort(v.begin(), v.end());
    return (int64_t)(std::unique(v.begin(), v.end()) - v.begin());
}

int ewpt_spectrum(ewpt_ctx* c, int32_t field, int32_t mode, int32_t nbins, double* k, double* sum, double* count,
                  double* mean, int32_t* nbins_out) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (field < EWPT_FIELD_B || field > EWPT_FIELD_HIGGS) return ewpt_fail(c, EWPT_ERR_ARG, "field %d unknown", field);
    if (mode != EWPT_SPEC_LOG && mode != EWPT_SPEC_UNIQUE) return ewpt_fail(c, EWPT_ERR_ARG, "mode %d unknown", mode);
    if (nbins < 1 || (mode == EWPT_SPEC_LOG && nbins > MAXSHELL))
        return ewpt_fail(c, EWPT_ERR_ARG, "nbins %d out of range", nbins);
    if (!k || !sum || !count || !mean) return ewpt_fail(c, EWPT_ERR_ARG, "output pointer is NULL");
    cudaSetDevice(c->p.device);
    const Grid& g = c->g;
    const int ncomp = field == EWPT_FIELD_HIGGS ? 4 : 3;
    const int nxh = g.nx / 2 + 1;
    const int64_t nh = (int64_t)nxh * g.ny * g.nz;
    int rc;
    if (!c->fft_ready) {
        cufftHandle plan;
        if (cufftPlan3d(&plan, g.nz, g.ny, g.nx, CUFFT_D2Z) != CUFFT_SUCCESS)
            return ewpt_fail(c, EWPT_ERR_CUFFT, "cufftPlan3d failed");
        c->fft_plan = (int)plan;
        rc = ewpt_cuda_check(c, cudaMalloc(&c->field3, (size_t)4 * g.S * 8), "spectrum fields");
        if (rc) return rc;
        rc = ewpt_cuda_check(c, cudaMalloc(&c->fft_out, (size_t)nh * sizeof(cufftDoubleComplex)), "spectrum fft");
        if (rc) return rc;
        c->fft_ready = 1;
    }
    if (cufftSetStream((cufftHandle)c->fft_plan, c->st) != CUFFT_SUCCESS)
        return ewpt_fail(c, EWPT_ERR_CUFFT, "cufftSetStream failed");
    const double* y;
    rc = ewpt_state64(c, &y);
    if (rc) return rc;
    const int which = field == EWPT_FIELD_B ? 0 : (field == EWPT_FIELD_B2 ? 1 : 2);
    cudaError_t e = launch_fields(g, c->p, y, which, c->field3, c->st);
    int nm = std::min(g.nx, std::min(g.ny, g.nz));
    const int nmax = nm / 2;
    const int64_t mmax_unique = ipow2(g.nx / 2) + ipow2(g.ny / 2) + ipow2(g.nz / 2);
    const int nblk = 4 * 152;
    // scratch: log mode partials [nblk][2][nbins] + result; unique mode [2][mmax+1]
    const size_t need = mode == EWPT_SPEC_LOG ? (size_t)nblk * 2 * nbins + 2 * nbins + (nbins + 1)
                                              : (size_t)2 * (mmax_unique + 1);
    double* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync(&scratch, need * 8 + 64, c->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, need * 8, c->st);
    std::vector<int64_t> thr;
    int64_t* dthr = nullptr;
    if (mode == EWPT_SPEC_LOG) {
        thr = ewpt_shell_thresholds(nmax, nbins);
        dthr = reinterpret_cast<int64_t*>(scratch + (size_t)nblk * 2 * nbins + 2 * nbins);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dthr, thr.data(), (nbins + 1) * 8, cudaMemcpyHostToDevice, c->st);
    }
    for (int comp = 0; comp < ncomp && e == cudaSuccess; ++comp) {
        double* f = c->field3 + (size_t)comp * g.S;
        if (cufftExecD2Z((cufftHandle)c->fft_plan, f, (cufftDoubleComplex*)c->fft_out) != CUFFT_SUCCESS) {
            cudaFreeAsync(scratch, c->st);
            return ewpt_fail(c, EWPT_ERR_CUFFT, "cufftExecD2Z failed");
        }
        if (mode == EWPT_SPEC_LOG)
            k_bin_log<<<nblk, SB, 0, c->st>>>(g.nx, g.ny, g.nz, nxh, (const cufftDoubleComplex*)c->fft_out, dthr,
                                              nbins, comp == 0, scratch);
        else
            k_bin_unique<<<nblk, SB, 0, c->st>>>(g.nx, g.ny, g.nz, nxh, (const cufftDoubleComplex*)c->fft_out,
                                                 mmax_unique, field == EWPT_FIELD_HIGGS, comp == 0, scratch,
                                                 scratch + mmax_unique + 1);
        e = cudaGetLastError();
    }
    std::vector<double> h;
    if (mode == EWPT_SPEC_LOG) {
        double* res = scratch + (size_t)nblk * 2 * nbins;
        if (e == cudaSuccess) k_bin_fold<<<(2 * nbins + 127) / 128, 128, 0, c->st>>>(scratch, nblk, nbins, res), e = cudaGetLastError();
        h.resize(2 * nbins);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), res, 2 * nbins * 8, cudaMemcpyDeviceToHost, c->st);
    } else {
        h.resize(2 * (mmax_unique + 1));
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), scratch, h.size() * 8, cudaMemcpyDeviceToHost, c->st);
    }
    if (scratch) cudaFreeAsync(scratch, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(c, e, "spectrum");
    if (rc) return rc;
    int nout = 0;
    if (mode == EWPT_SPEC_LOG) {
        const double lmax = std::log((double)nmax);
        for (int b = 0; b < nbins; ++b) {
            k[b] = std::exp(lmax * (b + 0.5) / nbins);
            sum[b] = h[b];
            count[b] = h[nbins + b];
            mean[b] = count[b] > 0 ? sum[b] / count[b] : 0.0;
        }
        nout = nbins;
    } else {
        for (int64_t m = 0; m <= mmax_unique && nout < nbins; ++m) {
            const double cnt = h[mmax_unique + 1 + m];
            if (cnt <= 0) continue;
            k[nout] = std::sqrt((double)m);
            sum[nout] = h[m];
            count[nout] = cnt;
            mean[nout] = h[m] / cnt;
            ++nout;
        }
    }
    if (nbins_out) *nbins_out = nout;
    return EWPT_OK;
}

}  // extern "C"

void ewpt_release_aux(ewpt_ctx* c) {
    if (c->fft_ready) cufftDestroy((cufftHandle)c->fft_plan);
    c->fft_ready = 0;
    cudaFree(c->field3);
    cudaFree(c->fft_out);
    cudaFree(c->red);
    cudaFree(c->dres);
    c->field3 = nullptr;
    c->fft_out = nullptr;
    c->red = nullptr;
    c->dres = nullptr;
}
