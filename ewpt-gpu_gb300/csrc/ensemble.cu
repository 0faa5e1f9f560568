// ensemble.cu -- batched ensembles of independent lattices of uneven sizes.
//
// All members' FP32-form states live in five shared buffers (y_hi, y_lo,
// kacc, xa, xb), member m's [36][S_m] block at element offset off_m.  A
// member table in device memory holds each member's geometry, couplings,
// stencil coefficients and time step.  One RK4 stage over the whole ensemble
// is ONE launch of a persistent kernel: a grid sized to the GPU's resident
// capacity walks a global list of (member, x-y tile, z plane) work items, so
// small and large members share the SMs without a launch per member.  The
// four stage launches of one step are captured once into a CUDA graph and
// replayed per step; per-member Jex/gamma live in the table, so changing
// them needs no re-capture.  The arithmetic per site is exactly that of the
// single-lattice FP32 form (same physics template and epilogue), so a member
// evolves identically to a single context with the same tiling mode.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "accessors.cuh"
#include "ewpt_ctx.cuh"

namespace {

struct EnsMember {
    int nx, ny, nz, tiles_x;
    int tiles_y, pad_;
    int64_t S, off, tile0;
    PhysCoef<float> pc;
    StencilCoef<float> sc;
    float h2, h1, w6, pad2_;
};

struct EnsBufs {
    float* yhi;
    float* ylo;
    float* kacc;
    float* xa;
    float* xb;
};

__device__ __forceinline__ int find_member(const EnsMember* __restrict__ tab, int n, int64_t w) {
    int lo = 0, hi = n;  // tab[lo].tile0 <= w < tab[hi].tile0
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&tab[mid].tile0) <= w)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

template <int STAGE, typename T>
struct EnsSink {
    int S, c;  // 36 S < 2^31 (checked at creation): 32-bit offsets within a member
    float* kacc;
    float* yhi;
    float* ylo;
    float* xn;
    T h, w6;
    const float* xin;  // stage input (for stage 1: y_hi)

    __device__ __forceinline__ static T rd(const float* p) {
        if constexpr (sizeof(T) == 8)
            return T(__ldg(reinterpret_cast<const float2*>(p)));
        else
            return T(__ldg(p));
    }
    __device__ __forceinline__ static void wr(float* p, const T& v) {
        if constexpr (sizeof(T) == 8)
            *reinterpret_cast<float2*>(p) = v.v;
        else
            *p = v;
    }
    __device__ __forceinline__ void operator()(int a, T r) const {
        const int q = a * S + c;
        if (STAGE == 1) {
            wr(kacc + q, r);
            wr(xn + q, T(rd(xin + q) + h * r));
        } else if (STAGE < 4) {
            wr(kacc + q, T(rd(kacc + q) + T(2.f) * r));
            wr(xn + q, T(rd(yhi + q) + h * r));
        } else {
            const T s = rd(kacc + q) + r;
            T hi = rd(yhi + q), lo = rd(ylo + q);
            acc_hilo(hi, lo, T(w6 * s));
            wr(yhi + q, hi);
            wr(ylo + q, lo);
        }
    }
};

template <typename T>
__device__ __forceinline__ PhysCoef<T> widen(const PhysCoef<float>& c) {
    return PhysCoef<T>{T(c.gw),   T(c.gy),    T(c.hgw),   T(c.hgy),   T(c.gp2),  T(c.omgp2), T(c.lam2),
                       T(c.vev2), T(c.bW),    T(c.bY),    T(c.bW2),   T(c.bY2),  T(c.hJex),  T(c.gam),
                       T(c.gg),   T(c.ggy),   T(c.lam2h), T(c.hJexh), T(c.gamh), T(c.ryw),   T(c.igw)};
}

template <int STAGE, bool BETA, bool PAIR>
__global__ void __launch_bounds__(128, 1) k_ens_stage(const EnsMember* __restrict__ tab, int nmem, int64_t ntiles,
                                                     EnsBufs b) {
    using T = typename std::conditional<PAIR, f2, float>::type;
    const float* xin = STAGE == 1 ? b.yhi : (STAGE == 3 ? b.xb : b.xa);
    float* xn = STAGE == 1 ? b.xa : (STAGE == 2 ? b.xb : b.xa);
    for (int64_t w = blockIdx.x; w < ntiles; w += gridDim.x) {
        const int m = find_member(tab, nmem, w);
        const EnsMember M = tab[m];
        int64_t t = w - M.tile0;
        const int tx = (int)(t % M.tiles_x);
        t /= M.tiles_x;
        const int ty = (int)(t % M.tiles_y);
        const int k = (int)(t / M.tiles_y);
        const int i = (tx * (int)blockDim.x + (int)threadIdx.x) * (PAIR ? 2 : 1);
        const int j = ty * (int)blockDim.y + (int)threadIdx.y;
        if (i >= M.nx || j >= M.ny) continue;
        const PhysCoef<T> pc = widen<T>(M.pc);
        EnsSink<STAGE, T> out{(int)M.S,     0,
                              b.kacc + M.off, b.yhi + M.off,
                              b.ylo + M.off, xn ? xn + M.off : nullptr,
                              T(STAGE == 3 ? M.h1 : M.h2), T(M.w6),
                              xin + M.off};
        if constexpr (PAIR) {
            PairAcc<SrcBase32<float>> A{{xin + M.off, (int)M.S}};
            A.place(i, j, k, M.nx, M.ny, M.nz);
            A.s = pair_stencil(M.sc);
            out.c = A.c;
            site_rates<f2, BETA>(A, pc, out);
        } else {
            SiteAcc<float, float, SrcBase32<float>> A{{xin + M.off, (int)M.S}};
            A.place(i, j, k, M.nx, M.ny, M.nz);
            A.s = M.sc;
            out.c = A.c;
            site_rates<float, BETA>(A, pc, out);
        }
    }
}

template <bool BETA, bool PAIR>
void occupancy_blocks(int* nb) {
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_ens_stage<2, BETA, PAIR>, 128, 0);
    *nb = a > 0 ? a : 1;
}

}  // namespace

struct ewpt_ens {
    int n = 0;
    int device = 0;
    cudaStream_t st = nullptr;
    std::vector<ewpt_params> mp;
    std::vector<EnsMember> tab;
    EnsMember* dtab = nullptr;
    EnsBufs b{};
    int64_t total = 0;  // sum of 36*S_m
    int64_t ntiles = 0;
    int bx = 8, by = 8, pair = 0;  // 8x8 pair-threads: the fastest shape for mixed 48-160 members
    bool beta = false;
    int grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t it = 0;
    std::map<std::tuple<int, int, int>, ewpt_ctx*> views;  // FP64 views for diagnostics / spectra
    std::string err;
};

static int ens_fail(ewpt_ens* e, int code, const char* msg) {
    if (e) e->err = msg;
    return ewpt_fail(nullptr, code, "%s", msg);
}

static int ens_cuda(ewpt_ens* e, cudaError_t ce, const char* what) {
    if (ce == cudaSuccess) return EWPT_OK;
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(ce));
    return ens_fail(e, ce == cudaErrorMemoryAllocation ? EWPT_ERR_OOM : EWPT_ERR_CUDA, buf);
}

// Lay out the tiles for the current tiling and (re)capture the step graph.
static int ens_plan(ewpt_ens* e) {
    int64_t t0 = 0;
    const int sx = e->pair ? 2 : 1;
    for (int m = 0; m < e->n; ++m) {
        EnsMember& M = e->tab[m];
        M.tiles_x = (M.nx + e->bx * sx - 1) / (e->bx * sx);
        M.tiles_y = (M.ny + e->by - 1) / e->by;
        M.tile0 = t0;
        t0 += (int64_t)M.tiles_x * M.tiles_y * M.nz;
    }
    e->ntiles = t0;
    cudaError_t ce = cudaMemcpyAsync(e->dtab, e->tab.data(), sizeof(EnsMember) * e->n, cudaMemcpyHostToDevice, e->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
    int rc = ens_cuda(e, ce, "ensemble table");
    if (rc) return rc;
    int dev_sms = 0, nb = 1;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, e->device);
    if (e->pair) {
        if (e->beta) occupancy_blocks<true, true>(&nb); else occupancy_blocks<false, true>(&nb);
    } else {
        if (e->beta) occupancy_blocks<true, false>(&nb); else occupancy_blocks<false, false>(&nb);
    }
    const int64_t cap = (int64_t)dev_sms * nb * std::max(1, 128 / (e->bx * e->by));
    e->grid = (int)std::min<int64_t>(cap, e->ntiles);
    if (e->exec) cudaGraphExecDestroy(e->exec), e->exec = nullptr;
    if (e->graph) cudaGraphDestroy(e->graph), e->graph = nullptr;
    ce = cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        const dim3 gr(e->grid), bl(e->bx, e->by);
#define EWPT_ENS_LAUNCH(BETA, PAIR)                                                                  \
    k_ens_stage<1, BETA, PAIR><<<gr, bl, 0, e->st>>>(e->dtab, e->n, e->ntiles, e->b);                 \
    k_ens_stage<2, BETA, PAIR><<<gr, bl, 0, e->st>>>(e->dtab, e->n, e->ntiles, e->b);                 \
    k_ens_stage<3, BETA, PAIR><<<gr, bl, 0, e->st>>>(e->dtab, e->n, e->ntiles, e->b);                 \
    k_ens_stage<4, BETA, PAIR><<<gr, bl, 0, e->st>>>(e->dtab, e->n, e->ntiles, e->b);
        if (e->beta && e->pair) { EWPT_ENS_LAUNCH(true, true) }
        else if (e->beta) { EWPT_ENS_LAUNCH(true, false) }
        else if (e->pair) { EWPT_ENS_LAUNCH(false, true) }
        else { EWPT_ENS_LAUNCH(false, false) }
#undef EWPT_ENS_LAUNCH
        cudaError_t le = cudaGetLastError();
        ce = cudaStreamEndCapture(e->st, &e->graph);
        if (ce == cudaSuccess) ce = le;
    }
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&e->exec, e->graph, 0);
    return ens_cuda(e, ce, "ensemble graph");
}

static void fill_coef(EnsMember& M, const ewpt_params& p, double Jex, double gam) {
    M.pc = make_phys<float>(p, Jex, gam);
    M.sc = make_stencil<float>(p.dx);
    M.h2 = (float)(p.dt / 2.);
    M.h1 = (float)p.dt;
    M.w6 = (float)(p.dt / 6.);
}

extern "C" {

int ewpt_ensemble_create(int32_t n, const ewpt_params* members, ewpt_ens** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n < 1 || !members) return ewpt_fail(nullptr, EWPT_ERR_ARG, "need at least one member");
    for (int m = 0; m < n; ++m) {
        int rc = ewpt_validate_params(&members[m], nullptr);
        if (rc) return rc;
        if (members[m].precision != EWPT_FP32)
            return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble members use the FP32 form (member %d)", m);
        if (36 * (int64_t)members[m].nx * members[m].ny * members[m].nz >= ((int64_t)1 << 31))
            return ewpt_fail(nullptr, EWPT_ERR_ARG,
                             "ensemble members need 36 nx ny nz < 2^31 (member %d); evolve larger lattices alone", m);
        if (members[m].device != members[0].device)
            return ewpt_fail(nullptr, EWPT_ERR_ARG, "all members must be on one device");
    }
    ewpt_ens* e = new ewpt_ens();
    e->n = n;
    e->device = members[0].device;
    e->mp.assign(members, members + n);
    e->tab.resize(n);
    int64_t off = 0;
    bool all_even = true;
    for (int m = 0; m < n; ++m) {
        const ewpt_params& p = members[m];
        EnsMember& M = e->tab[m];
        std::memset(&M, 0, sizeof M);
        M.nx = p.nx;
        M.ny = p.ny;
        M.nz = p.nz;
        M.S = (int64_t)p.nx * p.ny * p.nz;
        M.off = off;
        off += 36 * M.S;
        fill_coef(M, p, 0.0, 0.0);
        all_even = all_even && (p.nx % 2 == 0);
        e->beta = e->beta || p.beta_w != 0.0 || p.beta_y != 0.0;
    }
    e->total = off;
    e->pair = all_even ? 1 : 0;
    cudaError_t ce = cudaSetDevice(e->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking);
    float** bufs[] = {&e->b.yhi, &e->b.ylo, &e->b.kacc, &e->b.xa, &e->b.xb};
    for (float** p : bufs)
        if (ce == cudaSuccess) ce = cudaMalloc(p, (size_t)off * 4);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->dtab, sizeof(EnsMember) * n);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(e->b.yhi, 0, (size_t)off * 4, e->st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(e->b.ylo, 0, (size_t)off * 4, e->st);
    int rc = ens_cuda(nullptr, ce, "ensemble allocation");
    if (!rc) rc = ens_plan(e);
    if (rc) {
        ewpt_ensemble_destroy(e);
        return rc;
    }
    *out = e;
    return EWPT_OK;
}

int ewpt_ensemble_destroy(ewpt_ens* e) {
    if (!e) return EWPT_OK;
    cudaSetDevice(e->device);
    if (e->st) cudaStreamSynchronize(e->st);
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    for (auto& kv : e->views) ewpt_destroy(kv.second);
    cudaFree(e->b.yhi);
    cudaFree(e->b.ylo);
    cudaFree(e->b.kacc);
    cudaFree(e->b.xa);
    cudaFree(e->b.xb);
    cudaFree(e->dtab);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
    return EWPT_OK;
}

const char* ewpt_ensemble_last_error(const ewpt_ens* e) { return e ? e->err.c_str() : ewpt_last_error(nullptr); }

int32_t ewpt_ensemble_size(const ewpt_ens* e) { return e ? e->n : -1; }

static int ens_member_check(ewpt_ens* e, int32_t m) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    if (m < 0 || m >= e->n) return ens_fail(e, EWPT_ERR_ARG, "member index out of range");
    return EWPT_OK;
}

// FP64 view context holding one member's state (state buffer only).
static int ens_view(ewpt_ens* e, int32_t m, ewpt_ctx** out) {
    const ewpt_params& p = e->mp[m];
    const auto key = std::make_tuple(p.nx, p.ny, p.nz);
    auto it = e->views.find(key);
    ewpt_ctx* v = nullptr;
    if (it == e->views.end()) {
        ewpt_params q = p;
        q.precision = EWPT_FP64;
        int rc = ewpt_create_view(&q, &v);
        if (rc) return ens_fail(e, rc, ewpt_last_error(nullptr));
        e->views[key] = v;
    } else {
        v = it->second;
    }
    v->p = p;  // couplings / dt / theta_w of this member
    v->p.precision = EWPT_FP64;
    // join the member's compensated state into the view (after queued steps)
    cudaEvent_t ev;
    cudaError_t ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev, e->st);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(v->st, ev, 0);
    const EnsMember& M = e->tab[m];
    if (ce == cudaSuccess) ce = launch_fp32_join(v->g, plain_layout(v->g), Fp32State{e->b.yhi + M.off, e->b.ylo + M.off}, v->y, v->st);
    cudaEventDestroy(ev);
    int rc = ens_cuda(e, ce, "ensemble view");
    if (rc) return rc;
    *out = v;
    return EWPT_OK;
}

int ewpt_ensemble_set_state(ewpt_ens* e, int32_t m, const double* packed, int32_t on_device) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!packed) return ens_fail(e, EWPT_ERR_ARG, "state is NULL");
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v);
    if (rc) return rc;
    const EnsMember& M = e->tab[m];
    cudaError_t ce = cudaStreamSynchronize(v->st);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(v->y, packed, (size_t)36 * M.S * 8,
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, e->st);
    if (ce == cudaSuccess) ce = launch_fp32_split(v->g, plain_layout(v->g), v->y, Fp32State{e->b.yhi + M.off, e->b.ylo + M.off}, e->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
    return ens_cuda(e, ce, "ensemble set_state");
}

int ewpt_ensemble_get_state(ewpt_ens* e, int32_t m, double* packed, int32_t on_device) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!packed) return ens_fail(e, EWPT_ERR_ARG, "state is NULL");
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v);
    if (rc) return rc;
    cudaError_t ce = cudaMemcpyAsync(packed, v->y, (size_t)36 * e->tab[m].S * 8,
                                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, v->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(v->st);
    return ens_cuda(e, ce, "ensemble get_state");
}

int ewpt_ensemble_set_drive(ewpt_ens* e, int32_t m, double Jex, double gamma) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!std::isfinite(Jex) || !std::isfinite(gamma)) return ens_fail(e, EWPT_ERR_ARG, "non-finite Jex/gamma");
    fill_coef(e->tab[m], e->mp[m], Jex, gamma);
    cudaSetDevice(e->device);
    cudaError_t ce = cudaMemcpyAsync(&e->dtab[m], &e->tab[m], sizeof(EnsMember), cudaMemcpyHostToDevice, e->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
    return ens_cuda(e, ce, "ensemble set_drive");
}

int ewpt_ensemble_set_tiling(ewpt_ens* e, int32_t bx, int32_t by, int32_t pair) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    if (bx < 1 || by < 1 || bx * by > 128 || (bx * by) % 32 != 0)
        return ens_fail(e, EWPT_ERR_ARG, "tile: need whole warps and at most 128 threads");
    if (pair != 0 && pair != 1) return ens_fail(e, EWPT_ERR_ARG, "pair must be 0 or 1");
    if (pair)
        for (const auto& p : e->mp)
            if (p.nx % 2) return ens_fail(e, EWPT_ERR_ARG, "paired sites need an even nx in every member");
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->st);
    e->bx = bx;
    e->by = by;
    e->pair = pair;
    return ens_plan(e);
}

int ewpt_ensemble_step(ewpt_ens* e, int32_t nsteps) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    if (nsteps < 0) return ens_fail(e, EWPT_ERR_ARG, "nsteps < 0");
    cudaSetDevice(e->device);
    for (int s = 0; s < nsteps; ++s) {
        int rc = ens_cuda(e, cudaGraphLaunch(e->exec, e->st), "ensemble step");
        if (rc) return rc;
        ++e->it;
    }
    return EWPT_OK;
}

int ewpt_ensemble_sync(ewpt_ens* e) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    cudaSetDevice(e->device);
    return ens_cuda(e, cudaStreamSynchronize(e->st), "ensemble sync");
}

void* ewpt_ensemble_stream(ewpt_ens* e) { return e ? (void*)e->st : nullptr; }

int64_t ewpt_ensemble_sites(const ewpt_ens* e) { return e ? e->total / 36 : -1; }

int ewpt_ensemble_init_bubbles(ewpt_ens* e, int32_t m, int32_t nb, const double* bubbles, int32_t profile, double p0,
                               double p1) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (nb < 0 || (nb > 0 && !bubbles)) return ens_fail(e, EWPT_ERR_ARG, "bubble list");
    if (profile != EWPT_BUBBLE_REFERENCE && profile != EWPT_BUBBLE_TANH) return ens_fail(e, EWPT_ERR_ARG, "profile");
    cudaSetDevice(e->device);
    const ewpt_params& p = e->mp[m];
    const EnsMember& M = e->tab[m];
    const Grid g{p.nx, p.ny, p.nz, M.S};
    std::string err;
    rc = ewpt_launch_bubbles(g, p.dx, nb, bubbles, profile, profile == EWPT_BUBBLE_REFERENCE ? p.mH : p0, p1, p.vev,
                             nullptr, e->b.yhi + M.off, e->b.ylo + M.off, plain_layout(g), e->st, &err);
    if (rc) return ens_fail(e, rc, err.c_str());
    return EWPT_OK;
}

static int ens_thermal(ewpt_ens* e, int32_t m, double T, double mH, double mW, uint64_t seed, int gauss_iters) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    rc = ewpt_check_thermal(T, mH, mW);
    if (rc) return ens_fail(e, rc, ewpt_last_error(nullptr));
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v);
    if (rc) return rc;
    std::string err;
    // after the view's join (same stream)
    rc = ewpt_thermal_fill(v->g, v->p, T, mH, mW, seed, v->y, v->st, &err, gauss_iters);
    if (rc) return ens_fail(e, rc, ("init_thermal: " + err).c_str());
    const EnsMember& M = e->tab[m];
    cudaError_t ce =
        launch_fp32_split(v->g, plain_layout(v->g), v->y, Fp32State{e->b.yhi + M.off, e->b.ylo + M.off}, e->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
    return ens_cuda(e, ce, "ensemble init_thermal");
}

int ewpt_ensemble_init_thermal(ewpt_ens* e, int32_t m, double T, double mH, double mW, uint64_t seed) {
    return ens_thermal(e, m, T, mH, mW, seed, -1);
}

int ewpt_ensemble_init_thermal_gauss(ewpt_ens* e, int32_t m, double T, double mH, double mW, uint64_t seed,
                                     int32_t gauss_iters) {
    if (gauss_iters < 0) return ens_fail(e, EWPT_ERR_ARG, "gauss_iters < 0");
    return ens_thermal(e, m, T, mH, mW, seed, gauss_iters);
}

int ewpt_ensemble_diagnostics(ewpt_ens* e, int32_t m, double out[EWPT_NDIAG]) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!out) return ens_fail(e, EWPT_ERR_ARG, "out is NULL");
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v);
    if (rc) return rc;
    rc = ewpt_diagnostics(v, out);
    if (rc) e->err = v->err;
    return rc;
}

int ewpt_ensemble_spectrum(ewpt_ens* e, int32_t m, int32_t field, int32_t mode, int32_t nbins, double* k,
                           double* sum, double* count, double* mean, int32_t* nbins_out) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v);
    if (rc) return rc;
    rc = ewpt_spectrum(v, field, mode, nbins, k, sum, count, mean, nbins_out);
    if (rc) e->err = v->err;
    return rc;
}

}  // extern "C"
