// mlp.cu -- the learned surrogate: a 3-layer BF16 MLP (n_in -> width ->
// width -> n_out, GELU, FP32 accumulate) trained on the GPU with hand-written
// tensor-core forward/backward kernels and AdamW.
//
// GEMMs run on the 5th-generation tensor cores (tcgen05.mma kind::f16,
// BF16 x BF16 -> FP32 accumulated in tensor memory; k_gemm_tc): every
// product of the forward pass (X W^T), the weight gradients (dZ^T A) and the
// input gradients (dZ W).  Weights are held in FP32 (the
// optimizer's master copy) and in BF16 (the GEMM operand); activations and
// gradients enter the GEMMs as BF16, pre-activations and accumulations stay
// FP32.  This network has no counterpart in the reference: it maps early-time
// spectra of the evolution to late-time magnetic spectra for parameter
// sweeps, and the evolution itself stays the fallback and the reference answer.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "ewpt_ctx.cuh"

namespace {

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

struct GemmArgs {
    const __nv_bfloat16* A;
    const __nv_bfloat16* B;
    float* C;
    int M, N, K, lda, ldb, ldc;
    int transA, transB;
    long spin;  // polls before the commit wait gives up
};

__device__ __forceinline__ __nv_bfloat16 ldA(const GemmArgs& g, int m, int k) {
    if (m >= g.M || k >= g.K) return __float2bfloat16(0.f);
    return g.transA ? g.A[(int64_t)k * g.lda + m] : g.A[(int64_t)m * g.lda + k];
}
__device__ __forceinline__ __nv_bfloat16 ldB(const GemmArgs& g, int k, int n) {
    if (k >= g.K || n >= g.N) return __float2bfloat16(0.f);
    return g.transB ? g.B[(int64_t)n * g.ldb + k] : g.B[(int64_t)k * g.ldb + n];
}

// ---------------------------------------------------------------- tcgen05
// C[M x N] = op(A) op(B) on the 5th-generation tensor cores: one CTA of 4
// warps per 128 x 64 tile of C, the FP32 accumulator in tensor memory (64
// TMEM columns), K in slabs of 64.  Per slab the 128 threads gather op(A)
// (128 x 64) and op(B)^T (64 x 64) as BF16 into shared memory in the
// canonical K-major layout without swizzle -- 8-row x 16-byte core matrices,
// adjacent along K 128 bytes apart (LBO), 8-row groups 1024 bytes apart
// (SBO) -- (zero outside the matrices, any transposition done by the
// gather), then one thread issues four tcgen05.mma (M 128, N 64, K 16) and
// commits them to an mbarrier that every thread waits on before the slab is
// overwritten.  Finally each warp reads its 32 TMEM lanes (rows) with
// tcgen05.ld and writes C.  Every wait is bounded (g.spin polls, host-set
// by ewpt_mlp_set_wait_limit, default kTcSpin).  A wait that runs out in any
// thread ends the slab loop for the whole CTA (a block-wide vote, so every
// thread leaves the loop at the same barrier), sets g_tc_err and skips the
// remaining tensor-core work; before the TMEM columns are freed the CTA waits
// again, with the full kTcSpin limit, for the MMAs already committed.
constexpr int TC_M = 128, TC_N = 64, TC_K = 64;
constexpr long kTcSpin = 1L << 22;
__device__ int g_tc_err = 0;

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, LBO, SBO (bytes), version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, long spin) {
    for (long it = 0; it < spin; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__global__ void __launch_bounds__(128) k_gemm_tc(GemmArgs g) {
    __shared__ __align__(1024) uint8_t sa[TC_M * TC_K * 2];  // 16 KB
    __shared__ __align__(1024) uint8_t sb[TC_N * TC_K * 2];  // 8 KB
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * TC_N;
    const uint32_t ubar = tc_smem(&bar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                     "r"(TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    bool ok = true;
    const int nslab = (g.K + TC_K - 1) / TC_K;
    for (int ks = 0; ks < nslab && ok; ++ks) {
        const int k0 = ks * TC_K;
        // gather op(A): row m = tid, 8 chunks of 8 K-elements (one core-matrix row each)
        for (int kc = 0; kc < TC_K / 8; ++kc) {
            uint32_t w[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
                w[e] = pack_bf16(ldA(g, m0 + tid, k0 + 8 * kc + 2 * e), ldA(g, m0 + tid, k0 + 8 * kc + 2 * e + 1));
            const int off = ((tid >> 3) * (TC_K / 8) + kc) * 128 + (tid & 7) * 16;
            *reinterpret_cast<uint4*>(sa + off) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        // gather op(B)^T: row n, 8 chunks along K; 64 rows x 8 chunks over 128 threads
        for (int q = tid; q < TC_N * (TC_K / 8); q += 128) {
            const int n = q >> 3, kc = q & 7;
            uint32_t w[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
                w[e] = pack_bf16(ldB(g, k0 + 8 * kc + 2 * e, n0 + n), ldB(g, k0 + 8 * kc + 2 * e + 1, n0 + n));
            const int off = ((n >> 3) * (TC_K / 8) + kc) * 128 + (n & 7) * 16;
            *reinterpret_cast<uint4*>(sb + off) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t abase = tc_smem(sa), bbase = tc_smem(sb);
#pragma unroll
            for (int kk = 0; kk < TC_K / 16; ++kk) {
                // K = 16 is two core matrices along K: advance 2 x LBO
                const uint64_t ad = tc_desc(abase + kk * 256, 128, (TC_K / 8) * 128);
                const uint64_t bd = tc_desc(bbase + kk * 256, 128, (TC_K / 8) * 128);
                const uint32_t acc = (ks > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(tc_idesc(TC_M, TC_N)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(ubar)
                         : "memory");
        }
        const bool late = !tc_wait(ubar, ks & 1, g.spin);
        if (__syncthreads_or(late)) {
            // the MMAs of this slab still read shared memory and write TMEM:
            // let them finish before the CTA leaves the loop
            tc_wait(ubar, ks & 1, kTcSpin);
            ok = false;
            if (tid == 0) atomicExch(&g_tc_err, 1);
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < TC_N; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < g.M)
#pragma unroll
                for (int e = 0; e < 16; ++e)
                    if (n0 + c0 + e < g.N) g.C[(int64_t)row * g.ldc + n0 + c0 + e] = __uint_as_float(r[e]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// z += bias (in place, z keeps the pre-activation); act = bf16(gelu(z)) or bf16(z)
__global__ void k_bias_act(float* z, const float* __restrict__ bias, __nv_bfloat16* act, int B, int N, int apply) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)B * N;
         q += (int64_t)gridDim.x * blockDim.x) {
        const float v = z[q] + bias[q % N];
        z[q] = v;
        if (act) act[q] = __float2bfloat16(apply ? gelu(v) : v);
    }
}

__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* y, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        y[q] = __float2bfloat16(x[q]);
}

// dz = 2 (z - y)/(B N) (MSE); per-block partial loss sums
__global__ void k_mse(const float* __restrict__ z, const float* __restrict__ y, float* dzf, __nv_bfloat16* dzb,
                      int64_t n, float scale, float* part) {
    __shared__ float sh[256];
    float s = 0.f;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float d = z[q] - y[q];
        s += d * d;
        const float g = 2.f * d * scale;
        dzf[q] = g;
        dzb[q] = __float2bfloat16(g);
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// dz = da * gelu'(z)
__global__ void k_gelu_bwd(const float* __restrict__ da, const float* __restrict__ z, float* dzf, __nv_bfloat16* dzb,
                           int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float g = da[q] * gelu_grad(z[q]);
        dzf[q] = g;
        dzb[q] = __float2bfloat16(g);
    }
}

// db[n] = sum_b dz[b][n]
__global__ void k_colsum(const float* __restrict__ dz, float* db, int B, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dz[(int64_t)b * N + n];
    db[n] = s;
}

__global__ void k_adamw(float* w, const float* __restrict__ g, float* m, float* v, int64_t n, float lr, float b1,
                        float b2, float eps, float wd, float c1, float c2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float gq = g[q];
        const float mq = b1 * m[q] + (1.f - b1) * gq;
        const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        w[q] = w[q] - lr * ((mq / c1) / (sqrtf(vq / c2) + eps) + wd * w[q]);
    }
}

__global__ void k_sum_partials(const float* __restrict__ part, int n, float* out) {
    float s = 0.f;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
}

}  // namespace

struct ewpt_mlp {
    int nin = 0, width = 0, nout = 0, maxb = 0, device = 0;
    cudaStream_t st = nullptr;
    int64_t wait_polls = -1;  // limit of the GEMM's tensor-core waits in polls (< 0: default)
    int64_t np = 0;
    int64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16* pb = nullptr;  // bf16 copy of p
    float* xf = nullptr;          // [maxb][nin] input (f32)
    float* yf = nullptr;          // [maxb][nout] target
    __nv_bfloat16* x0 = nullptr;  // [maxb][nin]
    float *z1 = nullptr, *z2 = nullptr, *z3 = nullptr;
    __nv_bfloat16 *a1 = nullptr, *a2 = nullptr;
    float* da = nullptr;          // [maxb][max(width, nout)]
    float* dzf = nullptr;
    __nv_bfloat16* dzb = nullptr;
    float* part = nullptr;        // loss partials
    float* loss = nullptr;
    int64_t t = 0;
    std::string err;
};

namespace {

int mlp_fail(ewpt_mlp* n, int code, const char* msg) {
    if (n) n->err = msg;
    return ewpt_fail(nullptr, code, "%s", msg);
}

int mlp_cuda(ewpt_mlp* n, cudaError_t e, const char* what) {
    if (e == cudaSuccess) {
        // a bounded tensor-core wait that ran out (k_gemm_tc) invalidates the results
        int h = 0;
        if (cudaMemcpyFromSymbol(&h, g_tc_err, sizeof h) == cudaSuccess && h) {
            const int z = 0;
            cudaMemcpyToSymbol(g_tc_err, &z, sizeof z);
            return mlp_fail(n, EWPT_ERR_TIMEOUT, "a tensor-core wait in the MLP GEMM ran out (results invalid)");
        }
        return EWPT_OK;
    }
    std::string s = std::string(what) + ": " + cudaGetErrorString(e);
    return mlp_fail(n, e == cudaErrorMemoryAllocation ? EWPT_ERR_OOM : EWPT_ERR_CUDA, s.c_str());
}

cudaError_t gemm(const ewpt_mlp* n, const __nv_bfloat16* A, int lda, int transA, const __nv_bfloat16* B, int ldb,
                 int transB, float* C, int ldc, int M, int N, int K) {
    const cudaStream_t st = n->st;
    GemmArgs g{A, B, C, M, N, K, lda, ldb, ldc, transA, transB, n->wait_polls < 0 ? kTcSpin : (long)n->wait_polls};
    const dim3 gr((N + TC_N - 1) / TC_N, (M + TC_M - 1) / TC_M);
    k_gemm_tc<<<gr, 128, 0, st>>>(g);
    return cudaGetLastError();
}

const int kEW = 1216;  // elementwise grid

cudaError_t refresh_bf16(ewpt_mlp* n) {
    k_to_bf16<<<kEW, 256, 0, n->st>>>(n->p, n->pb, n->np);
    return cudaGetLastError();
}

// Forward pass on the batch already in n->xf; leaves z1, z2, z3, a1, a2.
cudaError_t forward(ewpt_mlp* n, int B) {
    cudaError_t e;
    k_to_bf16<<<kEW, 256, 0, n->st>>>(n->xf, n->x0, (int64_t)B * n->nin);
    e = gemm(n, n->x0, n->nin, 0, n->pb + n->oW1, n->nin, 1, n->z1, n->width, B, n->width, n->nin);
    if (e) return e;
    k_bias_act<<<kEW, 256, 0, n->st>>>(n->z1, n->p + n->ob1, n->a1, B, n->width, 1);
    e = gemm(n, n->a1, n->width, 0, n->pb + n->oW2, n->width, 1, n->z2, n->width, B, n->width, n->width);
    if (e) return e;
    k_bias_act<<<kEW, 256, 0, n->st>>>(n->z2, n->p + n->ob2, n->a2, B, n->width, 1);
    e = gemm(n, n->a2, n->width, 0, n->pb + n->oW3, n->width, 1, n->z3, n->nout, B, n->nout, n->width);
    if (e) return e;
    k_bias_act<<<kEW, 256, 0, n->st>>>(n->z3, n->p + n->ob3, nullptr, B, n->nout, 0);
    return cudaGetLastError();
}

// Loss and gradients into n->g (target batch in n->yf).
cudaError_t backward(ewpt_mlp* n, int B) {
    cudaError_t e;
    const int W = n->width, O = n->nout, I = n->nin;
    const int nb = 64;
    k_mse<<<nb, 256, 0, n->st>>>(n->z3, n->yf, n->dzf, n->dzb, (int64_t)B * O, 1.f / ((float)B * O), n->part);
    k_sum_partials<<<1, 1, 0, n->st>>>(n->part, nb, n->loss);
    // layer 3
    e = gemm(n, n->dzb, O, 1, n->a2, W, 0, n->g + n->oW3, W, O, W, B);  // dW3 = dZ3^T A2
    if (e) return e;
    k_colsum<<<(O + 127) / 128, 128, 0, n->st>>>(n->dzf, n->g + n->ob3, B, O);
    e = gemm(n, n->dzb, O, 0, n->pb + n->oW3, W, 0, n->da, W, B, W, O);  // dA2 = dZ3 W3
    if (e) return e;
    k_gelu_bwd<<<kEW, 256, 0, n->st>>>(n->da, n->z2, n->dzf, n->dzb, (int64_t)B * W);
    // layer 2
    e = gemm(n, n->dzb, W, 1, n->a1, W, 0, n->g + n->oW2, W, W, W, B);  // dW2 = dZ2^T A1
    if (e) return e;
    k_colsum<<<(W + 127) / 128, 128, 0, n->st>>>(n->dzf, n->g + n->ob2, B, W);
    e = gemm(n, n->dzb, W, 0, n->pb + n->oW2, W, 0, n->da, W, B, W, W);  // dA1 = dZ2 W2
    if (e) return e;
    k_gelu_bwd<<<kEW, 256, 0, n->st>>>(n->da, n->z1, n->dzf, n->dzb, (int64_t)B * W);
    // layer 1
    e = gemm(n, n->dzb, W, 1, n->x0, I, 0, n->g + n->oW1, I, W, I, B);  // dW1 = dZ1^T X0
    if (e) return e;
    k_colsum<<<(W + 127) / 128, 128, 0, n->st>>>(n->dzf, n->g + n->ob1, B, W);
    return cudaGetLastError();
}

int check_batch(ewpt_mlp* n, int B) {
    if (!n) return ewpt_fail(nullptr, EWPT_ERR_ARG, "mlp is NULL");
    if (B < 1 || B > n->maxb) return mlp_fail(n, EWPT_ERR_ARG, "batch size out of range (1..max_batch)");
    cudaSetDevice(n->device);
    return EWPT_OK;
}

cudaError_t upload(ewpt_mlp* n, float* dst, const float* src, int64_t count) {
    return cudaMemcpyAsync(dst, src, count * 4, cudaMemcpyHostToDevice, n->st);
}

}  // namespace

extern "C" {

int ewpt_mlp_create(int32_t n_in, int32_t width, int32_t n_out, int32_t max_batch, int32_t device, ewpt_mlp** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_in < 1 || width < 1 || n_out < 1 || max_batch < 1 || n_in > 65536 || width > 65536 || n_out > 65536)
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "bad MLP dimensions");
    ewpt_mlp* n = new ewpt_mlp();
    n->nin = n_in;
    n->width = width;
    n->nout = n_out;
    n->maxb = max_batch;
    n->device = device;
    n->oW1 = 0;
    n->ob1 = n->oW1 + (int64_t)width * n_in;
    n->oW2 = n->ob1 + width;
    n->ob2 = n->oW2 + (int64_t)width * width;
    n->oW3 = n->ob2 + width;
    n->ob3 = n->oW3 + (int64_t)n_out * width;
    n->np = n->ob3 + n_out;
    const int64_t wa = std::max(width, n_out);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking);
    auto A = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, n->st);
    };
    A((void**)&n->p, n->np * 4);
    A((void**)&n->g, n->np * 4);
    A((void**)&n->m, n->np * 4);
    A((void**)&n->v, n->np * 4);
    A((void**)&n->pb, n->np * 2);
    A((void**)&n->xf, (size_t)max_batch * n_in * 4);
    A((void**)&n->yf, (size_t)max_batch * n_out * 4);
    A((void**)&n->x0, (size_t)max_batch * n_in * 2);
    A((void**)&n->z1, (size_t)max_batch * width * 4);
    A((void**)&n->z2, (size_t)max_batch * width * 4);
    A((void**)&n->z3, (size_t)max_batch * n_out * 4);
    A((void**)&n->a1, (size_t)max_batch * width * 2);
    A((void**)&n->a2, (size_t)max_batch * width * 2);
    A((void**)&n->da, (size_t)max_batch * wa * 4);
    A((void**)&n->dzf, (size_t)max_batch * wa * 4);
    A((void**)&n->dzb, (size_t)max_batch * wa * 2);
    A((void**)&n->part, 64 * 4);
    A((void**)&n->loss, 4);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    int rc = mlp_cuda(nullptr, e, "mlp allocation");
    if (rc) {
        ewpt_mlp_destroy(n);
        return rc;
    }
    *out = n;
    return EWPT_OK;
}

int ewpt_mlp_destroy(ewpt_mlp* n) {
    if (!n) return EWPT_OK;
    cudaSetDevice(n->device);
    if (n->st) cudaStreamSynchronize(n->st);
    void* bufs[] = {n->p, n->g, n->m, n->v, n->pb, n->xf, n->yf, n->x0, n->z1, n->z2, n->z3,
                    n->a1, n->a2, n->da, n->dzf, n->dzb, n->part, n->loss};
    for (void* b : bufs) cudaFree(b);
    if (n->st) cudaStreamDestroy(n->st);
    delete n;
    return EWPT_OK;
}

const char* ewpt_mlp_last_error(const ewpt_mlp* n) { return n ? n->err.c_str() : ewpt_last_error(nullptr); }

int64_t ewpt_mlp_num_params(const ewpt_mlp* n) { return n ? n->np : -1; }

int ewpt_mlp_set_wait_limit(ewpt_mlp* n, int64_t polls) {
    if (!n) return ewpt_fail(nullptr, EWPT_ERR_ARG, "net is NULL");
    n->wait_polls = polls < 0 ? -1 : polls;
    return EWPT_OK;
}

int ewpt_mlp_set_params(ewpt_mlp* n, const float* params) {
    if (!n || !params) return ewpt_fail(nullptr, EWPT_ERR_ARG, "NULL argument");
    for (int64_t q = 0; q < n->np; ++q)
        if (!std::isfinite(params[q])) return mlp_fail(n, EWPT_ERR_ARG, "non-finite parameter");
    cudaSetDevice(n->device);
    cudaError_t e = cudaMemcpyAsync(n->p, params, n->np * 4, cudaMemcpyHostToDevice, n->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->m, 0, n->np * 4, n->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->v, 0, n->np * 4, n->st);
    if (e == cudaSuccess) e = refresh_bf16(n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    n->t = 0;
    return mlp_cuda(n, e, "mlp set_params");
}

int ewpt_mlp_get_params(ewpt_mlp* n, float* params) {
    if (!n || !params) return ewpt_fail(nullptr, EWPT_ERR_ARG, "NULL argument");
    cudaSetDevice(n->device);
    cudaError_t e = cudaMemcpyAsync(params, n->p, n->np * 4, cudaMemcpyDeviceToHost, n->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    return mlp_cuda(n, e, "mlp get_params");
}

int ewpt_mlp_forward(ewpt_mlp* n, const float* x, int32_t batch, float* y) {
    int rc = check_batch(n, batch);
    if (rc) return rc;
    if (!x || !y) return mlp_fail(n, EWPT_ERR_ARG, "NULL argument");
    cudaError_t e = upload(n, n->xf, x, (int64_t)batch * n->nin);
    if (e == cudaSuccess) e = forward(n, batch);
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, n->z3, (size_t)batch * n->nout * 4, cudaMemcpyDeviceToHost, n->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    return mlp_cuda(n, e, "mlp forward");
}

int ewpt_mlp_gradients(ewpt_mlp* n, const float* x, const float* y, int32_t batch, float* grads, float* loss) {
    int rc = check_batch(n, batch);
    if (rc) return rc;
    if (!x || !y || !grads) return mlp_fail(n, EWPT_ERR_ARG, "NULL argument");
    cudaError_t e = upload(n, n->xf, x, (int64_t)batch * n->nin);
    if (e == cudaSuccess) e = upload(n, n->yf, y, (int64_t)batch * n->nout);
    if (e == cudaSuccess) e = forward(n, batch);
    if (e == cudaSuccess) e = backward(n, batch);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grads, n->g, n->np * 4, cudaMemcpyDeviceToHost, n->st);
    float l = 0.f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, n->loss, 4, cudaMemcpyDeviceToHost, n->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    if (loss) *loss = l / ((float)batch * n->nout);
    return mlp_cuda(n, e, "mlp gradients");
}

int ewpt_mlp_train_step(ewpt_mlp* n, const float* x, const float* y, int32_t batch, float lr, float weight_decay,
                        float* loss) {
    int rc = check_batch(n, batch);
    if (rc) return rc;
    if (!x || !y) return mlp_fail(n, EWPT_ERR_ARG, "NULL argument");
    if (!std::isfinite(lr) || !std::isfinite(weight_decay)) return mlp_fail(n, EWPT_ERR_ARG, "non-finite lr/wd");
    cudaError_t e = upload(n, n->xf, x, (int64_t)batch * n->nin);
    if (e == cudaSuccess) e = upload(n, n->yf, y, (int64_t)batch * n->nout);
    if (e == cudaSuccess) e = forward(n, batch);
    if (e == cudaSuccess) e = backward(n, batch);
    n->t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->t), c2 = 1.f - std::pow(b2, (float)n->t);
    if (e == cudaSuccess) {
        k_adamw<<<kEW, 256, 0, n->st>>>(n->p, n->g, n->m, n->v, n->np, lr, b1, b2, 1e-8f, weight_decay, c1, c2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = refresh_bf16(n);
    float l = 0.f;
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(&l, n->loss, 4, cudaMemcpyDeviceToHost, n->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
    if (loss) *loss = l / ((float)batch * n->nout);
    return mlp_cuda(n, e, "mlp train_step");
}

}  // extern "C"
