// slab.cu -- z-slab domain decomposition of one periodic lattice.
//
// The reference splits its lattice over MPI ranks, one GPU each, and
// refreshes 3-plane ghost layers with host-staged MPI.Sendrecv! after every
// stage (update_halo!, boundary_x/y/z, gpu-kernels-rk4/main_rk4_multiple.jl:
// 69-212).  Here a lattice of nx x ny x nz sites is cut along z into slabs
// of nz_m planes.  A slab context holds its FP64 buffers (y, yn and the two
// stage inputs) as nx x ny x (nz_m + 6) planes per array: 3 ghost planes
// below the interior and 3 above.  Its stage kernels are the single
// lattice's k_stage_fp64 with the z neighbours read from the ghost planes
// (Grid::zg = 3) instead of wrapped, so a decomposed step gives the same
// bits as the undecomposed one.  Before every stage the ghost planes of
// that stage's input are filled from the neighbouring slabs: per face one
// strided copy of 36 arrays x 3 planes (cudaMemcpy2DAsync, a peer copy when
// the neighbour lives on another GPU).
//
//   ewpt_slabs_*            one process drives all slabs (one GPU or
//                           several); neighbour order comes from events.
//   ewpt_create_slab,       one slab per process (one rank per GPU): the
//   ewpt_slab_stage/pack/   caller moves the packed faces between ranks
//   unpack                  (ewpt/slabs.py does it with torch.distributed).
#include <cmath>
#include <string>
#include <vector>

#include "ewpt_ctx.cuh"

namespace {

constexpr int kZg = 3;  // ghost planes per z face (the 6th-order stencil's reach)

// Input buffer of stage s (1..4) of a step: y, X2, X3, X4.
double* stage_input(ewpt_ctx* c, int s) { return s == 1 ? c->y : s == 3 ? c->xb : c->xa; }

int64_t plane(const ewpt_ctx* c) { return (int64_t)c->g.nx * c->g.ny; }

// 36 arrays x 3 planes between two [36][S] buffers with independent plane offsets.
cudaError_t copy_planes(double* dst, int64_t dst_stride, int64_t dst_plane0, const double* src, int64_t src_stride,
                        int64_t src_plane0, int64_t plane_elems, cudaStream_t st) {
    return cudaMemcpy2DAsync(dst + dst_plane0 * plane_elems, (size_t)dst_stride * 8, src + src_plane0 * plane_elems,
                             (size_t)src_stride * 8, (size_t)kZg * plane_elems * 8, 36, cudaMemcpyDefault, st);
}

int slab_check(ewpt_ctx* c) {
    if (!c) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ctx is NULL");
    if (!c->slab) return ewpt_fail(c, EWPT_ERR_STATE, "not a slab context (ewpt_create_slab)");
    return EWPT_OK;
}

}  // namespace

// Copy the interior of a slab between its padded buffer and a packed
// [36][nx ny nz_m] buffer (host or device).
cudaError_t ewpt_slab_copy(ewpt_ctx* c, double* packed, bool to_dev, int32_t on_device) {
    const int64_t P = plane(c), n = P * c->g.nz;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice
                                          : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    double* dev = c->y + kZg * P;
    return to_dev ? cudaMemcpy2DAsync(dev, (size_t)c->g.S * 8, packed, (size_t)n * 8, (size_t)n * 8, 36, kind, c->st)
                  : cudaMemcpy2DAsync(packed, (size_t)n * 8, dev, (size_t)c->g.S * 8, (size_t)n * 8, 36, kind, c->st);
}

extern "C" {

int ewpt_create_slab(const ewpt_params* global, int32_t z0, int32_t nz_local, ewpt_ctx** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = ewpt_validate_params(global, nullptr);
    if (rc) return rc;
    if (global->precision != EWPT_FP64) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs need the FP64 form");
    if (global->stencil_order && global->stencil_order != 6)
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs need the 6th-order stencil (3 ghost planes)");
    if (nz_local < kZg || z0 < 0 || z0 + nz_local > global->nz)
        return ewpt_fail(nullptr, EWPT_ERR_ARG, "slab planes [%d, %d) of %d: need >= %d planes inside the lattice", z0,
                         z0 + nz_local, global->nz, kZg);
    ewpt_ctx* c = new ewpt_ctx();
    c->p = *global;
    c->p.stencil_order = 6;
    c->slab = true;
    c->z0 = z0;
    c->nz_global = global->nz;
    c->g = Grid{global->nx, global->ny, nz_local, (int64_t)global->nx * global->ny * (nz_local + 2 * kZg), kZg};
    cudaError_t e = cudaSetDevice(global->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    const size_t n = (size_t)36 * c->g.S;
    double** bufs[] = {&c->y, &c->yn, &c->xa, &c->xb};
    for (double** b : bufs) {
        if (e == cudaSuccess) e = cudaMalloc(b, n * 8);
        if (e == cudaSuccess) e = cudaMemsetAsync(*b, 0, n * 8, c->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    rc = ewpt_cuda_check(nullptr, e, "slab allocation");
    if (rc) {
        ewpt_destroy(c);
        return rc;
    }
    *out = c;
    return EWPT_OK;
}

int ewpt_slab_stage(ewpt_ctx* c, int32_t stage, double Jex, double gamma) {
    int rc = slab_check(c);
    if (rc) return rc;
    if (stage < 1 || stage > 4) return ewpt_fail(c, EWPT_ERR_ARG, "stage %d: 1..4", stage);
    if (!std::isfinite(Jex) || !std::isfinite(gamma)) return ewpt_fail(c, EWPT_ERR_ARG, "non-finite Jex/gamma");
    cudaSetDevice(c->p.device);
    rc = ewpt_cuda_check(c, launch_stage_fp64(c->g, c->tile, stage, c->y, c->yn, c->xa, c->xb, c->p, Jex, gamma, c->st),
                         "slab stage");
    if (rc == EWPT_OK && stage == 4) ++c->it;
    return rc;
}

int ewpt_slab_pack(ewpt_ctx* c, int32_t stage, double* lo, double* hi) {
    int rc = slab_check(c);
    if (rc) return rc;
    if (stage < 1 || stage > 4 || !lo || !hi) return ewpt_fail(c, EWPT_ERR_ARG, "stage 1..4 and two device buffers");
    cudaSetDevice(c->p.device);
    const int64_t P = plane(c), w = kZg * P;
    const double* b = stage_input(c, stage);
    cudaError_t e = copy_planes(lo, w, 0, b, c->g.S, kZg, P, c->st);
    if (e == cudaSuccess) e = copy_planes(hi, w, 0, b, c->g.S, c->g.nz, P, c->st);
    return ewpt_cuda_check(c, e, "slab pack");
}

int ewpt_slab_unpack(ewpt_ctx* c, int32_t stage, const double* below, const double* above) {
    int rc = slab_check(c);
    if (rc) return rc;
    if (stage < 1 || stage > 4 || !below || !above)
        return ewpt_fail(c, EWPT_ERR_ARG, "stage 1..4 and two device buffers");
    cudaSetDevice(c->p.device);
    const int64_t P = plane(c), w = kZg * P;
    double* b = stage_input(c, stage);
    cudaError_t e = copy_planes(b, c->g.S, 0, below, w, 0, P, c->st);
    if (e == cudaSuccess) e = copy_planes(b, c->g.S, c->g.nz + kZg, above, w, 0, P, c->st);
    return ewpt_cuda_check(c, e, "slab unpack");
}

}  // extern "C"

// ------------------------------------------------------------- slab group
struct ewpt_slabs {
    ewpt_params p{};
    std::vector<ewpt_ctx*> s;
    std::vector<cudaEvent_t> done;  // per slab: its last stage finished
    int64_t it = 0;
    std::string err;
};

namespace {

int slabs_fail(ewpt_slabs* G, int code, const std::string& msg) {
    if (G) G->err = msg;
    return ewpt_fail(nullptr, code, "%s", msg.c_str());
}

// Fill the ghost planes of every slab's stage-s input from its neighbours
// (periodic in z), after the neighbours' previous stage.  The copies run on
// the receiving slab's stream; that stream's next kernel follows them, and a
// neighbour's next write of the lent planes comes only after it has waited
// for this slab's following stage (the event chain of every exchange).
cudaError_t exchange(ewpt_slabs* G, int s) {
    const int n = (int)G->s.size();
    cudaError_t e = cudaSuccess;
    for (int m = 0; m < n && e == cudaSuccess; ++m) {
        cudaSetDevice(G->s[m]->p.device);
        e = cudaEventRecord(G->done[m], G->s[m]->st);
    }
    for (int m = 0; m < n && e == cudaSuccess; ++m) {
        ewpt_ctx* c = G->s[m];
        ewpt_ctx* lo = G->s[(m + n - 1) % n];
        ewpt_ctx* hi = G->s[(m + 1) % n];
        cudaSetDevice(c->p.device);
        e = cudaStreamWaitEvent(c->st, G->done[(m + n - 1) % n], 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->st, G->done[(m + 1) % n], 0);
        const int64_t P = plane(c);
        double* b = stage_input(c, s);
        // lower ghosts <- the top 3 interior planes of the slab below
        if (e == cudaSuccess) e = copy_planes(b, c->g.S, 0, stage_input(lo, s), lo->g.S, lo->g.nz, P, c->st);
        // upper ghosts <- the bottom 3 interior planes of the slab above
        if (e == cudaSuccess) e = copy_planes(b, c->g.S, c->g.nz + kZg, stage_input(hi, s), hi->g.S, kZg, P, c->st);
    }
    return e;
}

// J_ext and damp (main_rk4.jl:5154-5172), as ewpt_step applies them.
double jext(const ewpt_params& p, int64_t it) {
    return (((double)it * p.dt * p.mH <= p.t_sat) && p.thermal_init) ? p.mH * p.mH : 0.0;
}
double dampv(const ewpt_params& p, int64_t it) {
    return (((double)it * p.dt * p.mH < p.t_sat) && p.thermal_init) ? 0.0 : p.gamma_inp;
}

int slabs_steps(ewpt_slabs* G, int32_t nsteps, bool expl, double Jex, double gam) {
    if (!G) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs is NULL");
    if (nsteps < 0) return slabs_fail(G, EWPT_ERR_ARG, "nsteps < 0");
    if (expl && (!std::isfinite(Jex) || !std::isfinite(gam))) return slabs_fail(G, EWPT_ERR_ARG, "non-finite Jex/gamma");
    for (int32_t k = 0; k < nsteps; ++k) {
        const int64_t it = G->it + 1;
        const double J = expl ? Jex : jext(G->p, it), D = expl ? gam : dampv(G->p, it);
        for (int s = 1; s <= 4; ++s) {
            cudaError_t e = exchange(G, s);
            for (size_t m = 0; m < G->s.size() && e == cudaSuccess; ++m) {
                ewpt_ctx* c = G->s[m];
                cudaSetDevice(c->p.device);
                e = launch_stage_fp64(c->g, c->tile, s, c->y, c->yn, c->xa, c->xb, c->p, J, D, c->st);
            }
            if (e != cudaSuccess) return slabs_fail(G, EWPT_ERR_CUDA, std::string("slab step: ") + cudaGetErrorString(e));
        }
        G->it = it;
        for (ewpt_ctx* c : G->s) c->it = it;
    }
    return EWPT_OK;
}

// Copy a packed global [36][nx ny nz] state into (to_dev) or out of the slabs.
int slabs_copy(ewpt_slabs* G, double* packed, bool to_dev, int32_t on_device) {
    if (!G) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs is NULL");
    if (!packed) return slabs_fail(G, EWPT_ERR_ARG, "state buffer is NULL");
    const int64_t S = (int64_t)G->p.nx * G->p.ny * G->p.nz;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDefault : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    cudaError_t e = cudaSuccess;
    for (ewpt_ctx* c : G->s) {
        if (e != cudaSuccess) break;
        cudaSetDevice(c->p.device);
        const int64_t P = plane(c), n = P * c->g.nz;
        double* g0 = packed + (int64_t)c->z0 * P;
        double* d0 = c->y + kZg * P;
        e = to_dev ? cudaMemcpy2DAsync(d0, (size_t)c->g.S * 8, g0, (size_t)S * 8, (size_t)n * 8, 36, kind, c->st)
                   : cudaMemcpy2DAsync(g0, (size_t)S * 8, d0, (size_t)c->g.S * 8, (size_t)n * 8, 36, kind, c->st);
    }
    for (ewpt_ctx* c : G->s) {
        cudaSetDevice(c->p.device);
        const cudaError_t es = cudaStreamSynchronize(c->st);
        if (e == cudaSuccess) e = es;
    }
    if (e != cudaSuccess) return slabs_fail(G, EWPT_ERR_CUDA, std::string("slab state copy: ") + cudaGetErrorString(e));
    if (to_dev) {
        G->it = 0;
        for (ewpt_ctx* c : G->s) c->it = 0;
    }
    return EWPT_OK;
}

}  // namespace

extern "C" {

int ewpt_slabs_create(const ewpt_params* global, int32_t n, const int32_t* nz_local, const int32_t* devices,
                      ewpt_slabs** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = ewpt_validate_params(global, nullptr);
    if (rc) return rc;
    if (n < 1) return ewpt_fail(nullptr, EWPT_ERR_ARG, "need at least one slab");
    std::vector<int> nz(n);
    int64_t total = 0;
    for (int m = 0; m < n; ++m) {
        nz[m] = nz_local ? nz_local[m] : global->nz / n + (m < global->nz % n ? 1 : 0);
        total += nz[m];
    }
    if (total != global->nz) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slab planes sum to %lld, not nz = %d",
                                              (long long)total, global->nz);
    ewpt_slabs* G = new ewpt_slabs();
    G->p = *global;
    int z0 = 0;
    for (int m = 0; m < n; ++m) {
        ewpt_params q = *global;
        if (devices) q.device = devices[m];
        ewpt_ctx* c = nullptr;
        rc = ewpt_create_slab(&q, z0, nz[m], &c);
        if (rc) {
            ewpt_slabs_destroy(G);
            return rc;
        }
        G->s.push_back(c);
        cudaEvent_t ev = nullptr;
        cudaSetDevice(q.device);
        const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            ewpt_slabs_destroy(G);
            return ewpt_cuda_check(nullptr, e, "slab event");
        }
        G->done.push_back(ev);
        z0 += nz[m];
    }
    *out = G;
    return EWPT_OK;
}

int ewpt_slabs_destroy(ewpt_slabs* G) {
    if (!G) return EWPT_OK;
    for (size_t m = 0; m < G->s.size(); ++m) {
        cudaSetDevice(G->s[m]->p.device);
        if (m < G->done.size()) cudaEventDestroy(G->done[m]);
        ewpt_destroy(G->s[m]);
    }
    delete G;
    return EWPT_OK;
}

const char* ewpt_slabs_last_error(const ewpt_slabs* G) { return G ? G->err.c_str() : ewpt_last_error(nullptr); }

int32_t ewpt_slabs_count(const ewpt_slabs* G) { return G ? (int32_t)G->s.size() : -1; }

int ewpt_slabs_set_state(ewpt_slabs* G, const double* packed, int32_t on_device) {
    return slabs_copy(G, const_cast<double*>(packed), true, on_device);
}

int ewpt_slabs_get_state(ewpt_slabs* G, double* packed, int32_t on_device) {
    return slabs_copy(G, packed, false, on_device);
}

int ewpt_slabs_set_tiling(ewpt_slabs* G, int32_t bx, int32_t by, int32_t reg) {
    if (!G) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs is NULL");
    for (ewpt_ctx* c : G->s) {
        const int rc = ewpt_set_tiling(c, bx, by, reg, 0);
        if (rc) return slabs_fail(G, rc, c->err);
    }
    return EWPT_OK;
}

int ewpt_slabs_step(ewpt_slabs* G, int32_t nsteps) { return slabs_steps(G, nsteps, false, 0.0, 0.0); }

int ewpt_slabs_step_explicit(ewpt_slabs* G, int32_t nsteps, double Jex, double gamma) {
    return slabs_steps(G, nsteps, true, Jex, gamma);
}

int ewpt_slabs_sync(ewpt_slabs* G) {
    if (!G) return ewpt_fail(nullptr, EWPT_ERR_ARG, "slabs is NULL");
    for (ewpt_ctx* c : G->s) {
        cudaSetDevice(c->p.device);
        const cudaError_t e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) return slabs_fail(G, EWPT_ERR_CUDA, std::string("slab sync: ") + cudaGetErrorString(e));
    }
    return EWPT_OK;
}

void* ewpt_slabs_stream(ewpt_slabs* G, int32_t m) {
    return G && m >= 0 && m < (int32_t)G->s.size() ? (void*)G->s[m]->st : nullptr;
}

}  // extern "C"
