// probe.cu -- measured FP64 peak of the GPU, the denominator of the FP64
// stage kernels' compute roofline.
//
// The FP64 form is bound by the FP64 pipe, not by HBM, so its roofline needs
// the pipe's own peak.  k_fp64_peak keeps eight independent fused
// multiply-add chains per thread on every SM (enough in flight to cover the
// DFMA latency) and ewpt_fp64_peak times it with CUDA events: FLOP/s =
// 2 x DFMAs / time.  No counterpart in the reference.
#include "ewpt_ctx.cuh"

namespace {

constexpr int kChains = 8;

__device__ double g_probe_sink;

__global__ void __launch_bounds__(256) k_fp64_peak(int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    // a store no input reaches (a = 1 - 2^-30, b small: |x| stays < 1e6), so the chains stay live
    if (s == 123456789.0) g_probe_sink = s;
}

}  // namespace

extern "C" int ewpt_fp64_peak(int32_t device, double* flop_per_s, double* seconds) {
    if (!flop_per_s) return ewpt_fail(nullptr, EWPT_ERR_ARG, "flop_per_s is NULL");
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess) e = cudaSetDevice(device);
    if (e != cudaSuccess) return ewpt_cuda_check(nullptr, e, "fp64 peak: device");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = 4 * (sms > 0 ? sms : 1), threads = 256, iters = 20000;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    if (e == cudaSuccess) {
        const double a = 1.0 - 1.0 / (1 << 30), b = 1e-9;
        k_fp64_peak<<<blocks, threads, 0, st>>>(iters / 4, a, b);  // warm-up
        cudaEventRecord(e0, st);
        k_fp64_peak<<<blocks, threads, 0, st>>>(iters, a, b);
        cudaEventRecord(e1, st);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaSetDevice(prev);
    int rc = ewpt_cuda_check(nullptr, e, "fp64 peak");
    if (rc) return rc;
    const double dfma = (double)blocks * threads * kChains * iters;
    *flop_per_s = 2.0 * dfma / (ms * 1e-3);
    if (seconds) *seconds = ms * 1e-3;
    return EWPT_OK;
}
