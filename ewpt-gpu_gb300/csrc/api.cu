// api.cu -- the C ABI of libewpt (declared in include/ewpt.h).
//
// A context owns the device state of one periodic lattice and one CUDA
// stream.  Host <-> device copies are explicit (ewpt_set_state /
// ewpt_get_state); stepping, diagnostics and spectra run on the stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "ewpt_ctx.cuh"
#include "stencil_n.cuh"

static thread_local std::string g_err = "";

int ewpt_fail(ewpt_ctx* ctx, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->err = buf;
    else
        g_err = buf;
    return code;
}

int ewpt_cuda_check(ewpt_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return EWPT_OK;
    if (e == cudaErrorMemoryAllocation)
        return ewpt_fail(ctx, EWPT_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return ewpt_fail(ctx, EWPT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ewpt_validate_params(const ewpt_params* p, ewpt_ctx* ctx) {
    if (!p) return ewpt_fail(ctx, EWPT_ERR_ARG, "params is NULL");
    if (p->nx < 7 || p->ny < 7 || p->nz < 7)
        return ewpt_fail(ctx, EWPT_ERR_ARG, "lattice %dx%dx%d: each axis needs >= 7 sites (3-site stencil halo)",
                         p->nx, p->ny, p->nz);
    if ((int64_t)p->nx * p->ny * p->nz > (int64_t)INT32_MAX)
        return ewpt_fail(ctx, EWPT_ERR_ARG, "lattice too large: nx*ny*nz must be < 2^31");
    if (p->precision != EWPT_FP64 && p->precision != EWPT_FP32 && p->precision != EWPT_DF64)
        return ewpt_fail(ctx, EWPT_ERR_ARG, "precision %d unknown", p->precision);
    {
        const int ord = p->stencil_order ? p->stencil_order : 6;
        const int R = stencil_radius(ord);
        if (R == 0) return ewpt_fail(ctx, EWPT_ERR_ARG, "stencil order %d unknown (2, 6, 8, 10 or 12)", ord);
        if (ord != 6 && p->precision != EWPT_FP64)
            return ewpt_fail(ctx, EWPT_ERR_ARG, "stencil order %d needs the FP64 form", ord);
        if (p->nx < 2 * R + 1 || p->ny < 2 * R + 1 || p->nz < 2 * R + 1)
            return ewpt_fail(ctx, EWPT_ERR_ARG, "stencil order %d needs >= %d sites per axis", ord, 2 * R + 1);
    }
    if (p->precision == EWPT_FP32 &&
        ghost_layout(Grid{p->nx, p->ny, p->nz, (int64_t)p->nx * p->ny * p->nz}).P + 64 > (int64_t)INT32_MAX)
        return ewpt_fail(ctx, EWPT_ERR_ARG, "lattice too large for the FP32 form's padded arrays (< 2^31 cells)");
    const double v[] = {p->dx, p->dt, p->gw, p->gy, p->gp2, p->lambda, p->vev, p->theta_w,
                        p->beta_w, p->beta_y, p->gamma_inp, p->mH, p->t_sat};
    for (double x : v)
        if (!std::isfinite(x)) return ewpt_fail(ctx, EWPT_ERR_ARG, "non-finite parameter");
    if (!(p->dx > 0)) return ewpt_fail(ctx, EWPT_ERR_ARG, "dx must be > 0");
    if (p->gw == 0.0)
        return ewpt_fail(ctx, EWPT_ERR_ARG, "gw must be nonzero (the stage kernels sum the SU(2) terms over g)");
    if (!(p->dt > 0)) return ewpt_fail(ctx, EWPT_ERR_ARG, "dt must be > 0");
    return EWPT_OK;
}

extern "C" {

int ewpt_params_default(ewpt_params* p, int32_t n) {
    if (!p) return ewpt_fail(nullptr, EWPT_ERR_ARG, "params is NULL");
    std::memset(p, 0, sizeof *p);
    p->nx = p->ny = p->nz = n;
    p->precision = EWPT_FP64;
    p->dx = 0.25;
    p->dt = p->dx / 10.0;
    p->gw = 0.65;
    p->theta_w = std::asin(std::sqrt(0.22));
    p->gy = p->gw * std::tan(p->theta_w);
    p->gp2 = 0.99;
    p->lambda = 0.129;
    p->vev = 1.0;
    p->beta_w = 0.0;
    p->beta_y = 0.0;
    p->gamma_inp = 0.0;
    p->mH = 2.0 * std::sqrt(p->lambda) * p->vev;
    p->t_sat = 2.0;
    p->thermal_init = 0;
    p->device = 0;
    p->stencil_order = 6;
    return EWPT_OK;
}

const char* ewpt_last_error(const ewpt_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

int ewpt_create(const ewpt_params* p, ewpt_ctx** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = ewpt_validate_params(p, nullptr);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return ewpt_fail(nullptr, EWPT_ERR_CUDA, "no CUDA device available");
    if (p->device < 0 || p->device >= ndev)
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "device %d out of range (%d devices)", p->device, ndev);
    ewpt_ctx* c = new ewpt_ctx();
    c->p = *p;
    if (!c->p.stencil_order) c->p.stencil_order = 6;
    c->g.nx = p->nx;
    c->g.ny = p->ny;
    c->g.nz = p->nz;
    c->g.S = (int64_t)p->nx * p->ny * p->nz;
    c->it = 0;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    rc = ewpt_cuda_check(nullptr, e, "stream");
    if (rc) {
        delete c;
        return rc;
    }
    const size_t n = (size_t)36 * c->g.S;
    if (p->precision == EWPT_FP64 || p->precision == EWPT_DF64) {
        e = cudaMalloc(&c->y, n * 8);
        if (e == cudaSuccess) e = cudaMalloc(&c->yn, n * 8);
        if (e == cudaSuccess) e = cudaMalloc(&c->xa, n * 8);
        if (e == cudaSuccess) e = cudaMalloc(&c->xb, n * 8);
        if (e == cudaSuccess && p->precision == EWPT_DF64) e = cudaMalloc(&c->ddcur, (size_t)12 * c->g.S * 8);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->y, 0, n * 8, c->st);
    } else {
        // ghosted layout; zero everything so the ghost cells no kernel writes
        // (the box edges, never read by a stencil) hold finite values
        c->lay = ghost_layout(c->g);
        const size_t m = (size_t)36 * c->lay.P + 32;
        float** bufs[] = {&c->y32.hi, &c->y32.lo, &c->w32.kacc, &c->w32.xa, &c->w32.xb};
        e = cudaSuccess;
        for (float** b : bufs) {
            if (e == cudaSuccess) e = cudaMalloc(b, m * 4);
            if (e == cudaSuccess) e = cudaMemsetAsync(*b, 0, m * 4, c->st);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(nullptr, e, "state allocation");
    if (rc) {
        ewpt_destroy(c);
        return rc;
    }
    *out = c;
    return EWPT_OK;
}

int ewpt_create_view(const ewpt_params* p, ewpt_ctx** out) {
    int rc = ewpt_validate_params(p, nullptr);
    if (rc) return rc;
    ewpt_ctx* c = new ewpt_ctx();
    c->p = *p;
    if (!c->p.stencil_order) c->p.stencil_order = 6;
    c->p.precision = EWPT_FP64;
    c->g = Grid{p->nx, p->ny, p->nz, (int64_t)p->nx * p->ny * p->nz};
    c->view = true;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->y, (size_t)36 * c->g.S * 8);
    rc = ewpt_cuda_check(nullptr, e, "view allocation");
    if (rc) {
        ewpt_destroy(c);
        return rc;
    }
    *out = c;
    return EWPT_OK;
}

int ewpt_destroy(ewpt_ctx* c) {
    if (!c) return EWPT_OK;
    cudaSetDevice(c->p.device);
    if (c->st) cudaStreamSynchronize(c->st);
    ewpt_release_aux(c);
    cudaFree(c->y);
    cudaFree(c->yn);
    cudaFree(c->xa);
    cudaFree(c->xb);
    cudaFree(c->ddcur);
    ewpt_tma_release(c);
    cudaFree(c->y32.hi);
    cudaFree(c->y32.lo);
    cudaFree(c->w32.kacc);
    cudaFree(c->w32.xa);
    cudaFree(c->w32.xb);
    cudaFree(c->scratch64);
    for (cudaStream_t s : c->io_st)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t ev : c->io_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return EWPT_OK;
}

// Device buffer holding the packed FP64 state (for FP32 contexts, a staging
// buffer that split/join convert through).
int ewpt_staging64(ewpt_ctx* c, double** out, bool in) {
    if (c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "slab contexts take packed states (ewpt_set_state_packed)");
    if (c->p.precision == EWPT_FP64 || (in && c->p.precision == EWPT_DF64)) {
        *out = c->y;  // DF64: converted in place after the upload
        return EWPT_OK;
    }
    int rc = ewpt_ensure_scratch64(c);
    if (rc) return rc;
    *out = c->scratch64;
    return EWPT_OK;
}

// Copy the 36 arrays between the caller's pointers and a [36][S] buffer,
// Host <-> device copies of a state: one cudaMemcpyAsync per run of arrays
// that lie back to back in the caller's memory (a packed state is one run).
// A host run of more than kChunkMin bytes is cut into kChunks pieces copied
// concurrently on the context's stream and kChunks - 1 side streams (one
// DMA engine each), joined back into the context's stream by events.
constexpr int kChunks = 4;
constexpr size_t kChunkMin = (size_t)64 << 20;

static cudaError_t io_streams(ewpt_ctx* c) {
    cudaError_t e = cudaSuccess;
    for (cudaStream_t& s : c->io_st)
        if (!s && e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    for (cudaEvent_t& ev : c->io_ev)
        if (!ev && e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    return e;
}

static cudaError_t copy_chunked(ewpt_ctx* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    cudaError_t e = io_streams(c);
    if (e == cudaSuccess) e = cudaEventRecord(c->io_ev[0], c->st);  // fork after the work queued so far
    const size_t piece = (bytes / kChunks + 4095) & ~(size_t)4095;
    for (int i = 0; i < kChunks && e == cudaSuccess; ++i) {
        const size_t off = (size_t)i * piece;
        if (off >= bytes) break;
        const size_t n = std::min(piece, bytes - off);
        cudaStream_t s = i == 0 ? c->st : c->io_st[i - 1];
        if (i > 0) e = cudaStreamWaitEvent(s, c->io_ev[0], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, n, kind, s);
        if (e == cudaSuccess && i > 0) e = cudaEventRecord(c->io_ev[i], s);
        if (e == cudaSuccess && i > 0) e = cudaStreamWaitEvent(c->st, c->io_ev[i], 0);  // join
    }
    return e;
}

static cudaError_t copy_runs(ewpt_ctx* c, double* dev, const double* const* arrays, int64_t S, bool to_dev,
                             int32_t on_device) {
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice
                                          : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    cudaError_t e = cudaSuccess;
    for (int a = 0; a < 36 && e == cudaSuccess;) {
        int b = a + 1;
        while (b < 36 && arrays[b] == arrays[b - 1] + S) ++b;
        const size_t bytes = (size_t)(b - a) * S * 8;
        double* d = dev + (size_t)a * S;
        void* dst = to_dev ? (void*)d : (void*)const_cast<double*>(arrays[a]);
        const void* src = to_dev ? (const void*)arrays[a] : (const void*)d;
        e = (!on_device && bytes > kChunkMin) ? copy_chunked(c, dst, src, bytes, kind)
                                              : cudaMemcpyAsync(dst, src, bytes, kind, c->st);
        a = b;
    }
    return e;
}

int ewpt_set_state(ewpt_ctx* c, const double* const arrays[EWPT_NARR], int32_t on_device) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "slab contexts take packed states (ewpt_set_state_packed)");
    if (!arrays) return ewpt_fail(c, EWPT_ERR_ARG, "arrays is NULL");
    for (int a = 0; a < 36; ++a)
        if (!arrays[a]) return ewpt_fail(c, EWPT_ERR_ARG, "arrays[%d] is NULL", a);
    cudaSetDevice(c->p.device);
    double* dst;
    int rc = ewpt_staging64(c, &dst, true);
    if (rc) return rc;
    cudaError_t e = copy_runs(c, dst, arrays, c->g.S, true, on_device);
    if (e == cudaSuccess) e = ewpt_commit_staged(c, dst);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    return ewpt_cuda_check(c, e, "set_state");
}

cudaError_t ewpt_commit_staged(ewpt_ctx* c, const double* staged) {
    if (c->p.precision == EWPT_FP32) return launch_fp32_split(c->g, c->lay, staged, c->y32, c->st);
    if (c->p.precision == EWPT_DF64) return launch_to_dd(36 * c->g.S, c->y, c->st);
    return cudaSuccess;
}

int ewpt_get_state(ewpt_ctx* c, double* const arrays[EWPT_NARR], int32_t on_device) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "slab contexts give packed states (ewpt_get_state_packed)");
    if (!arrays) return ewpt_fail(c, EWPT_ERR_ARG, "arrays is NULL");
    for (int a = 0; a < 36; ++a)
        if (!arrays[a]) return ewpt_fail(c, EWPT_ERR_ARG, "arrays[%d] is NULL", a);
    cudaSetDevice(c->p.device);
    double* src;
    int rc = ewpt_staging64(c, &src, false);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    if (c->p.precision == EWPT_FP32) e = launch_fp32_join(c->g, c->lay, c->y32, src, c->st);
    if (c->p.precision == EWPT_DF64) e = launch_from_dd(36 * c->g.S, c->y, src, c->st);
    if (e == cudaSuccess) e = copy_runs(c, src, arrays, c->g.S, false, on_device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(c, e, "get_state");
    return rc ? rc : ewpt_tma_check(c);
}

int ewpt_set_state_packed(ewpt_ctx* c, const double* buf, int32_t on_device) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!buf) return ewpt_fail(c, EWPT_ERR_ARG, "buf is NULL");
    if (c->slab) {
        cudaSetDevice(c->p.device);
        cudaError_t e = ewpt_slab_copy(c, const_cast<double*>(buf), true, on_device);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        c->it = 0;
        return ewpt_cuda_check(c, e, "slab set_state");
    }
    const double* a[36];
    for (int q = 0; q < 36; ++q) a[q] = buf + (size_t)q * c->g.S;
    return ewpt_set_state(c, a, on_device);
}

int ewpt_get_state_packed(ewpt_ctx* c, double* buf, int32_t on_device) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!buf) return ewpt_fail(c, EWPT_ERR_ARG, "buf is NULL");
    if (c->slab) {
        cudaSetDevice(c->p.device);
        cudaError_t e = ewpt_slab_copy(c, buf, false, on_device);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        return ewpt_cuda_check(c, e, "slab get_state");
    }
    double* a[36];
    for (int q = 0; q < 36; ++q) a[q] = buf + (size_t)q * c->g.S;
    return ewpt_get_state(c, a, on_device);
}

// J_ext and damp (main_rk4.jl:5154-5172).
static double jext_of(const ewpt_params& p, int64_t it) {
    return (((double)it * p.dt * p.mH <= p.t_sat) && p.thermal_init) ? p.mH * p.mH : 0.0;
}
static double damp_of(const ewpt_params& p, int64_t it) {
    return (((double)it * p.dt * p.mH < p.t_sat) && p.thermal_init) ? 0.0 : p.gamma_inp;
}

static int do_steps(ewpt_ctx* c, int32_t nsteps, bool expl, double Jex, double gam) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    if (c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "a slab steps stage by stage between ghost exchanges");
    if (nsteps < 0) return ewpt_fail(c, EWPT_ERR_ARG, "nsteps < 0");
    if (expl && (!std::isfinite(Jex) || !std::isfinite(gam)))
        return ewpt_fail(c, EWPT_ERR_ARG, "non-finite Jex/gamma");
    cudaSetDevice(c->p.device);
    for (int32_t s = 0; s < nsteps; ++s) {
        const int64_t it = c->it + 1;
        const double J = expl ? Jex : jext_of(c->p, it);
        const double G = expl ? gam : damp_of(c->p, it);
        cudaError_t e;
        if (c->p.precision == EWPT_FP64 && c->p.stencil_order != 6)
            e = launch_step_fp64_order(c->g, c->tile, c->y, c->yn, c->xa, c->xb, c->p, J, G, c->st);
        else if (c->p.precision == EWPT_FP64)
            e = launch_step_fp64(c->g, c->tile, c->y, c->yn, c->xa, c->xb, c->p, J, G, c->st);
        else if (c->p.precision == EWPT_DF64)
            e = launch_step_dd(c->g, c->tile, c->y, c->yn, c->xa, c->xb, c->ddcur, c->p, J, G, c->st);
        else if (c->tile.pair == 2)
            e = launch_step_fp32_tma(c, J, G);
        else
            e = (c->tile.pair && c->g.nx % 2 == 0)
                    ? launch_step_fp32_pair(c->g, c->lay, c->tile, c->y32, c->w32, c->p, J, G, c->st, c->fp32_comp)
                    : launch_step_fp32(c->g, c->lay, c->tile, c->y32, c->w32, c->p, J, G, c->st);
        int rc = ewpt_cuda_check(c, e, "step launch");
        if (rc) return rc;
        c->it = it;
    }
    return EWPT_OK;
}

int ewpt_step(ewpt_ctx* c, int32_t nsteps) { return do_steps(c, nsteps, false, 0.0, 0.0); }

// ---- host-to-host steps
// True when [p, p + bytes) is page-locked host memory (cudaHostAlloc or
// cudaHostRegister), which asynchronous copies can overlap with kernels.
static bool pinned_host(const void* p, size_t bytes) {
    const char* q[2] = {static_cast<const char*>(p), static_cast<const char*>(p) + bytes - 1};
    for (const char* x : q) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, x) != cudaSuccess) {
            cudaGetLastError();  // not a sticky error: clear it
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

// Upload (FP64 form, 6th-order stencils, pinned buffers): the state goes up
// in nwin windows of z planes, each window's 36 array pieces spread over
// the four io streams.  Stage 1 of the first step runs on the planes whose
// 3-plane neighbourhood has arrived while the next windows are in flight;
// stage 4 of the last step runs window by window, and each finished window
// goes down while the next is computed.  Every site sees the arithmetic of
// a whole-lattice launch, so the result is the one of set_state_packed +
// step + get_state_packed, bit for bit.
constexpr int kHostWindows = 8;  // windows per host step: min(8, nz / 16), at least 2

static int step_host_overlapped(ewpt_ctx* c, const double* in, double* out, int32_t nsteps) {
    const Grid& g = c->g;
    const int nz = g.nz, nio = 4;
    const int nwin = std::max(2, std::min(kHostWindows, nz / 16));
    const int64_t S = g.S, A = (int64_t)g.nx * g.ny;
    int zw[kHostWindows + 1];
    for (int w = 0; w <= nwin; ++w) zw[w] = (int)((int64_t)nz * w / nwin);
    cudaError_t e = io_streams(c);
    // the io streams start after the work queued on the context's stream
    auto fork = [&]() {
        if (e == cudaSuccess) e = cudaEventRecord(c->io_ev[4], c->st);
        for (int i = 0; i < nio && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(c->io_st[i], c->io_ev[4], 0);
    };
    // the context's stream waits for every copy queued so far
    auto join = [&]() {
        for (int i = 0; i < nio && e == cudaSuccess; ++i) {
            e = cudaEventRecord(c->io_ev[i], c->io_st[i]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(c->st, c->io_ev[i], 0);
        }
    };
    auto copy_window = [&](int w, bool up) {
        const int64_t off = zw[w] * A;
        const size_t bytes = (size_t)(zw[w + 1] - zw[w]) * A * sizeof(double);
        for (int a = 0; a < 36 && e == cudaSuccess; ++a) {
            double* dev = c->y + a * S + off;
            const int64_t h = a * S + off;
            e = up ? cudaMemcpyAsync(dev, in + h, bytes, cudaMemcpyHostToDevice, c->io_st[a % nio])
                   : cudaMemcpyAsync(out + h, dev, bytes, cudaMemcpyDeviceToHost, c->io_st[a % nio]);
        }
    };
    auto stage = [&](int s, int k0, int k1, double J, double G) {
        if (e == cudaSuccess)
            e = launch_stage_fp64_planes(g, c->tile, s, k0, k1, c->y, c->yn, c->xa, c->xb, c->p, J, G, c->st);
    };
    for (int32_t s = 0; s < nsteps && e == cudaSuccess; ++s) {
        const int64_t it = c->it + 1 + s;
        const double J = jext_of(c->p, it), G = damp_of(c->p, it);
        if (s == 0) {
            fork();
            int lo = 3;  // planes [3, lo) have had stage 1
            for (int w = 0; w < nwin; ++w) {
                copy_window(w, true);
                join();
                const int hi = w == nwin - 1 ? nz : zw[w + 1] - 3;
                if (hi > lo) {
                    stage(1, lo, hi, J, G);
                    lo = hi;
                }
            }
            stage(1, 0, 3, J, G);  // their lower neighbours wrap to the top planes
        } else {
            stage(1, 0, nz, J, G);
        }
        stage(2, 0, nz, J, G);
        stage(3, 0, nz, J, G);
        if (s < nsteps - 1) {
            stage(4, 0, nz, J, G);
            continue;
        }
        for (int w = 0; w < nwin; ++w) {
            stage(4, zw[w], zw[w + 1], J, G);
            fork();
            copy_window(w, false);
        }
        join();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {  // drain what was queued before reporting
        for (cudaStream_t st : c->io_st)
            if (st) cudaStreamSynchronize(st);
        cudaStreamSynchronize(c->st);
        return ewpt_cuda_check(c, e, "step_host");
    }
    c->it += nsteps;
    return EWPT_OK;
}

int ewpt_step_host(ewpt_ctx* c, const double* state_in, double* state_out, int32_t nsteps) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!state_in || !state_out) return ewpt_fail(c, EWPT_ERR_ARG, "state_in or state_out is NULL");
    if (nsteps < 0) return ewpt_fail(c, EWPT_ERR_ARG, "nsteps < 0");
    if (c->view) return ewpt_fail(c, EWPT_ERR_STATE, "this context is a read-only view");
    if (c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "a slab steps stage by stage between ghost exchanges");
    cudaSetDevice(c->p.device);
    const size_t bytes = (size_t)36 * c->g.S * sizeof(double);
    if (nsteps > 0 && c->p.precision == EWPT_FP64 && c->p.stencil_order == 6 && c->g.nz >= 16 &&
        pinned_host(state_in, bytes) && pinned_host(state_out, bytes))
        return step_host_overlapped(c, state_in, state_out, nsteps);
    int rc = ewpt_set_state_packed(c, state_in, 0);
    if (!rc) rc = ewpt_step(c, nsteps);
    if (!rc) rc = ewpt_get_state_packed(c, state_out, 0);
    return rc;
}

int ewpt_step_explicit(ewpt_ctx* c, int32_t nsteps, double Jex, double gamma) {
    return do_steps(c, nsteps, true, Jex, gamma);
}

int64_t ewpt_iteration(const ewpt_ctx* c) { return c ? c->it : -1; }

int ewpt_set_fp32_compensated(ewpt_ctx* c, int32_t on) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (c->p.precision != EWPT_FP32) return ewpt_fail(c, EWPT_ERR_ARG, "the compensated mode is an FP32-form mode");
    if (on && (c->tile.pair != 1 || c->g.nx % 2 != 0))
        return ewpt_fail(c, EWPT_ERR_ARG, "the compensated mode runs two sites per thread: set a tiling with pair = 1");
    c->fp32_comp = on != 0;
    return EWPT_OK;
}

int32_t ewpt_get_fp32_compensated(const ewpt_ctx* c) { return c && c->fp32_comp ? 1 : 0; }

int ewpt_set_tiling(ewpt_ctx* c, int32_t bx, int32_t by, int32_t reg, int32_t pair) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (c->fp32_comp && pair != 1)
        return ewpt_fail(c, EWPT_ERR_ARG, "the compensated mode runs two sites per thread (pair = 1)");
    if (pair == 2) {
        // TMA-staged shared-memory tiles of bx x by x reg sites (FP32 form)
        if (bx != 32 || (by != 2 && by != 4) || reg != 4)
            return ewpt_fail(c, EWPT_ERR_ARG, "TMA tiles: bx = 32, by in {2, 4}, reg (the z extent) = 4");
        if (c->p.precision != EWPT_FP32) return ewpt_fail(c, EWPT_ERR_ARG, "TMA tiles need the FP32 form");
        int rc = ewpt_tma_prepare(c, by, reg);
        if (rc) return rc;
        // the other FP32 kernels leave the x ghost cells stale; the TMA boxes read them
        rc = ewpt_cuda_check(c, launch_ghost_fill(c->g, c->lay, c->y32.hi, c->st, true), "ghost fill");
        if (rc) return rc;
        c->tile = Tiling{bx, by, reg, pair};
        return EWPT_OK;
    }
    if (reg < 0 || reg > 2) return ewpt_fail(c, EWPT_ERR_ARG, "register variant %d unknown (0..2)", reg);
    if (bx < 1 || by < 1 || bx * by > tiling_max_threads(reg) || (bx * by) % 32 != 0)
        return ewpt_fail(c, EWPT_ERR_ARG, "tile %dx%d: need whole warps and at most %d threads for variant %d", bx, by,
                         tiling_max_threads(reg), reg);
    if (pair != 0 && pair != 1) return ewpt_fail(c, EWPT_ERR_ARG, "pair must be 0, 1 or 2");
    if (pair && c->g.nx % 2 != 0) return ewpt_fail(c, EWPT_ERR_ARG, "paired sites need an even nx");
    c->tile = Tiling{bx, by, reg, pair};
    return EWPT_OK;
}

int ewpt_set_wait_limit(ewpt_ctx* c, int64_t polls) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    c->wait_polls = polls < 0 ? -1 : polls;
    ewpt_tma_set_spin(c);
    return EWPT_OK;
}

int ewpt_get_tiling(const ewpt_ctx* c, int32_t* bx, int32_t* by, int32_t* reg, int32_t* pair) {
    if (!c || !bx || !by || !reg || !pair) return ewpt_fail(nullptr, EWPT_ERR_ARG, "NULL argument");
    *bx = c->tile.bx;
    *by = c->tile.by;
    *reg = c->tile.reg;
    *pair = c->tile.pair;
    return EWPT_OK;
}

int ewpt_sync(ewpt_ctx* c) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    cudaSetDevice(c->p.device);
    int rc = ewpt_cuda_check(c, cudaStreamSynchronize(c->st), "sync");
    return rc ? rc : ewpt_tma_check(c);
}

void* ewpt_stream(ewpt_ctx* c) { return c ? (void*)c->st : nullptr; }

int ewpt_rk4_rates(const ewpt_params* p, const double* const in[EWPT_NARR], double* const out[EWPT_NARR],
                   double Jex, double gamma, void* stream) {
    int rc = ewpt_validate_params(p, nullptr);
    if (rc) return rc;
    if (!in || !out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "in/out is NULL");
    Ptr36 I;
    MPtr36 O;
    for (int a = 0; a < 36; ++a) {
        if (!in[a] || !out[a]) return ewpt_fail(nullptr, EWPT_ERR_ARG, "array %d is NULL", a);
        I.p[a] = in[a];
        O.p[a] = out[a];
    }
    for (int a = 0; a < 36; ++a)
        for (int b = 0; b < 36; ++b)
            if ((const void*)in[a] == (const void*)out[b])
                return ewpt_fail(nullptr, EWPT_ERR_ARG, "in[%d] aliases out[%d]", a, b);
    if (!std::isfinite(Jex) || !std::isfinite(gamma)) return ewpt_fail(nullptr, EWPT_ERR_ARG, "non-finite Jex/gamma");
    Grid g{p->nx, p->ny, p->nz, (int64_t)p->nx * p->ny * p->nz};
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess)
        e = (p->stencil_order && p->stencil_order != 6)
                ? launch_rates_fp64_order(g, I, O, *p, Jex, gamma, (cudaStream_t)stream)
                : launch_rates_fp64(g, I, O, *p, Jex, gamma, (cudaStream_t)stream);
    return ewpt_cuda_check(nullptr, e, "rk4_rates");
}

}  // extern "C"
