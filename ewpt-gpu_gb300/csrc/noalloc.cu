// noalloc.cu -- snapshot diagnostics that allocate nothing.
//
// ewpt_diagnostics needs scratch memory for its per-block partial sums and
// gets it with cudaMalloc on first use.  Some callers cannot allow that: a
// host whose device memory is owned by another allocator's pool (a Julia
// CUDA.jl or PyTorch process that has reserved the device), a caller that
// must not grow its device footprint once a run has started, or code that
// must not hit the driver's allocator in the middle of a time-critical loop.
// This variant keeps its scratch in a fixed file-scope device array instead.
//
// The array is sized for EWPT_NOALLOC_MAX_TILES partial rows of kRowLen
// doubles, one row per 32x4-site x-y tile of the lattice, plus the final
// row: (4096 * 32 + 32) * 8 = 1,048,832 bytes.  Every GPU that loads the
// library holds it until the process exits.  Calls share the array: two
// calls whose kernels overlap on the GPU (on different streams, or from
// different host threads) race on it.
#include <cstdio>

#include "ewpt_ctx.cuh"

#define EWPT_NOALLOC_MAX_TILES 4096

cudaError_t launch_diag_bounded(const Grid& g, const ewpt_params& p, const double* y, double* part,
                                int64_t max_rows, double* dres, cudaStream_t st);
int64_t diag_tiles_xy(const Grid& g);
int diag_nred();
void diag_finish_row(const ewpt_params& p, int64_t S, const double* r, double* out);

namespace {

constexpr int kRowLen = 32;  // >= the reduction row length of diag.cu (22)
constexpr int64_t kScratch = (int64_t)EWPT_NOALLOC_MAX_TILES * kRowLen + kRowLen;

// The scratch.  In host code this name is only a stand-in for the device
// symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kScratch];

// Device address of the scratch on the current device.  Looked up on every
// call (it is not a stream operation and costs microseconds): a cached
// address would go stale if the caller reset the device or tore down its
// primary context, which reloads the module at a new address.
int scratch_address(int dev, double** out) {
    double* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        return ewpt_fail(nullptr, EWPT_ERR_CUDA, "cudaGetSymbolAddress(noalloc scratch) on device %d: %s", dev,
                         cudaGetErrorString(e));
    *out = ptr;
    return EWPT_OK;
}

// The diagnostics on the current device (the caller's device is restored by
// the entry point below).
int diagnostics_noalloc_on(const ewpt_params* p, const Grid& g, const double* state, double* out, cudaStream_t st) {
    double* scratch = nullptr;
    int rc = scratch_address(p->device, &scratch);
    if (rc) return rc;
    double* part = scratch;
    double* res = scratch + (int64_t)EWPT_NOALLOC_MAX_TILES * kRowLen;
    // Every block writes its whole partial row and the final kernel reads
    // only those rows, so what an earlier call left in the array is never
    // read and nothing needs clearing.
    cudaError_t e =
        launch_diag_bounded(g, *p, state, part, (int64_t)EWPT_NOALLOC_MAX_TILES * kRowLen / diag_nred(), res, st);
    double r[kRowLen];
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, res, (size_t)diag_nred() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rc = ewpt_cuda_check(nullptr, e, "diagnostics_noalloc");
    if (rc) return rc;
    diag_finish_row(*p, g.S, r, out);
    for (int q = 0; q < EWPT_NDIAG; ++q)
        if (!(out[q] == out[q]) || out[q] - out[q] != 0.0)
            return ewpt_fail(nullptr, EWPT_ERR_NONFINITE, "non-finite diagnostic column %d", q);
    return EWPT_OK;
}

}  // namespace

extern "C" int ewpt_diagnostics_noalloc(const ewpt_params* p, const double* state, double out[EWPT_NDIAG],
                                        void* stream) {
    int rc = ewpt_validate_params(p, nullptr);
    if (rc) return rc;
    if (!state || !out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "state/out is NULL");
    if (diag_nred() > kRowLen) return ewpt_fail(nullptr, EWPT_ERR_STATE, "reduction row longer than scratch rows");
    const Grid g{p->nx, p->ny, p->nz, (int64_t)p->nx * p->ny * p->nz};
    const int64_t tiles = diag_tiles_xy(g);
    if (tiles > EWPT_NOALLOC_MAX_TILES)
        return ewpt_fail(nullptr, EWPT_ERR_ARG,
                         "lattice %dx%d needs %lld x-y tiles of 32x4 sites; ewpt_diagnostics_noalloc holds at most %d "
                         "(use ewpt_diagnostics for larger lattices)",
                         p->nx, p->ny, (long long)tiles, EWPT_NOALLOC_MAX_TILES);
    // the caller's current device is put back on every path below: a Julia
    // or PyTorch host thread keeps the device it had chosen
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return ewpt_cuda_check(nullptr, e, "noalloc get device");
    e = cudaSetDevice(p->device);
    if (e != cudaSuccess) return ewpt_cuda_check(nullptr, e, "noalloc set device");
    rc = diagnostics_noalloc_on(p, g, state, out, (cudaStream_t)stream);
    e = cudaSetDevice(prev);
    if (rc == EWPT_OK && e != cudaSuccess) rc = ewpt_cuda_check(nullptr, e, "noalloc restore device");
    return rc;
}
