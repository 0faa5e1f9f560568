// ensemble.cu -- batched ensembles of independent lattices of uneven sizes.
//
// Each member is an ordinary FP32-form context (ghosted layout, the paired
// or one-site stage kernels of a single lattice, with their L2 prefetches
// and chunked block walk), so a member evolves exactly like a single context
// with the same tiling.  What the ensemble adds is the schedule: one RK4
// step of every member is ONE CUDA graph, captured once from the ensemble's
// stream and forked into one branch per member (each branch the member's
// four stage launches and ghost refreshes, on the member's stream, joined
// back at the end).  The branches are independent, so the GPU runs the
// members' kernels concurrently: the blocks of small members fill the SMs
// next to the large ones and no member's tail idles the GPU.  Replaying the
// graph costs one launch per step for the whole ensemble.  Per-member
// Jex/gamma are launch parameters of the branch: changing them marks the
// graph for capture before the next step.
//
// State I/O, initial conditions, diagnostics and spectra of a member run on
// the ensemble's stream through an FP64 view context per member size (one
// [36][S] FP64 buffer shared by the members of that size), so they are
// ordered with the queued steps and need no per-member FP64 storage.
#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "ewpt_ctx.cuh"

struct ewpt_ens {
    int n = 0;
    int device = 0;
    cudaStream_t st = nullptr;
    std::vector<ewpt_params> mp;
    std::vector<ewpt_ctx*> mem;      // one FP32-form context per member
    std::vector<double> jex, gam;    // per-member drive (default 0, 0)
    Tiling tile{16, 8, 2, 0};
    bool dirty = true;               // the step graph must be captured again
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t it = 0;
    int64_t sites = 0;
    std::map<std::tuple<int, int, int>, ewpt_ctx*> views;  // FP64 views per member size
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

// Capture one step of every member into the graph: fork from the ensemble's
// stream into the members' streams, each member's step there, join back.
static int ens_capture(ewpt_ens* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec), e->exec = nullptr;
    if (e->graph) cudaGraphDestroy(e->graph), e->graph = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal);
    cudaError_t le = cudaSuccess;
    if (ce == cudaSuccess) {
        le = cudaEventRecord(e->fork, e->st);
        for (int m = 0; m < e->n && le == cudaSuccess; ++m) {
            ewpt_ctx* c = e->mem[m];
            le = cudaStreamWaitEvent(c->st, e->fork, 0);
            if (le == cudaSuccess)
                le = c->tile.pair ? launch_step_fp32_pair(c->g, c->lay, c->tile, c->y32, c->w32, c->p, e->jex[m],
                                                          e->gam[m], c->st)
                                  : launch_step_fp32(c->g, c->lay, c->tile, c->y32, c->w32, c->p, e->jex[m],
                                                     e->gam[m], c->st);
            if (le == cudaSuccess) le = cudaEventRecord(e->join[m], c->st);
            if (le == cudaSuccess) le = cudaStreamWaitEvent(e->st, e->join[m], 0);
        }
        ce = cudaStreamEndCapture(e->st, &e->graph);
        if (ce == cudaSuccess) ce = le;
    }
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&e->exec, e->graph, 0);
    int rc = ens_cuda(e, ce, "ensemble graph");
    if (!rc) e->dirty = false;
    return rc;
}

extern "C" {

int ewpt_ensemble_create(int32_t n, const ewpt_params* members, ewpt_ens** out) {
    if (!out) return ewpt_fail(nullptr, EWPT_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n < 1 || !members) return ewpt_fail(nullptr, EWPT_ERR_ARG, "need at least one member");
    bool all_even = true;
    for (int m = 0; m < n; ++m) {
        int rc = ewpt_validate_params(&members[m], nullptr);
        if (rc) return rc;
        if (members[m].precision != EWPT_FP32)
            return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble members use the FP32 form (member %d)", m);
        if (members[m].device != members[0].device)
            return ewpt_fail(nullptr, EWPT_ERR_ARG, "all members must be on one device");
        all_even = all_even && members[m].nx % 2 == 0;
    }
    ewpt_ens* e = new ewpt_ens();
    e->n = n;
    e->device = members[0].device;
    e->mp.assign(members, members + n);
    e->jex.assign(n, 0.0);
    e->gam.assign(n, 0.0);
    e->tile = Tiling{16, 8, 2, all_even ? 1 : 0};
    cudaError_t ce = cudaSetDevice(e->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    e->join.assign(n, nullptr);
    for (int m = 0; m < n && ce == cudaSuccess; ++m) ce = cudaEventCreateWithFlags(&e->join[m], cudaEventDisableTiming);
    int rc = ens_cuda(nullptr, ce, "ensemble stream");
    for (int m = 0; m < n && !rc; ++m) {
        ewpt_ctx* c = nullptr;
        rc = ewpt_create(&members[m], &c);  // zero state, ghosted FP32 buffers
        if (!rc) {
            c->tile = e->tile;
            e->mem.push_back(c);
            e->sites += c->g.S;
        }
    }
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
    for (auto& kv : e->views) {
        kv.second->st = nullptr;  // the ensemble's stream, destroyed below
        ewpt_destroy(kv.second);
    }
    for (ewpt_ctx* c : e->mem) ewpt_destroy(c);
    for (cudaEvent_t ev : e->join)
        if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
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

// FP64 view of member m's size holding its state (joined after the steps
// queued on the ensemble's stream); the view's work runs on the ensemble's
// stream too.
static int ens_view(ewpt_ens* e, int32_t m, ewpt_ctx** out, bool join = true) {
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
        // the view works on the ensemble's stream (its own stream is idle)
        cudaStreamDestroy(v->st);
        v->st = e->st;
    } else {
        v = it->second;
    }
    v->p = p;  // couplings / dt / theta_w of this member
    v->p.precision = EWPT_FP64;
    if (join) {
        const ewpt_ctx* c = e->mem[m];
        int rc = ens_cuda(e, launch_fp32_join(v->g, c->lay, c->y32, v->y, e->st), "ensemble view");
        if (rc) return rc;
    }
    *out = v;
    return EWPT_OK;
}

int ewpt_ensemble_set_state(ewpt_ens* e, int32_t m, const double* packed, int32_t on_device) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!packed) return ens_fail(e, EWPT_ERR_ARG, "state is NULL");
    cudaSetDevice(e->device);
    ewpt_ctx* v;
    rc = ens_view(e, m, &v, false);
    if (rc) return rc;
    ewpt_ctx* c = e->mem[m];
    cudaError_t ce = cudaMemcpyAsync(v->y, packed, (size_t)36 * c->g.S * 8,
                                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, e->st);
    if (ce == cudaSuccess) ce = launch_fp32_split(c->g, c->lay, v->y, c->y32, e->st);
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
    cudaError_t ce = cudaMemcpyAsync(packed, v->y, (size_t)36 * e->mem[m]->g.S * 8,
                                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, e->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
    return ens_cuda(e, ce, "ensemble get_state");
}

int ewpt_ensemble_set_drive(ewpt_ens* e, int32_t m, double Jex, double gamma) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (!std::isfinite(Jex) || !std::isfinite(gamma)) return ens_fail(e, EWPT_ERR_ARG, "non-finite Jex/gamma");
    if (e->jex[m] != Jex || e->gam[m] != gamma) e->dirty = true;
    e->jex[m] = Jex;
    e->gam[m] = gamma;
    return EWPT_OK;
}

int ewpt_ensemble_set_tiling(ewpt_ens* e, int32_t bx, int32_t by, int32_t pair) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    if (bx < 1 || by < 1 || bx * by > 128 || (bx * by) % 32 != 0)
        return ens_fail(e, EWPT_ERR_ARG, "tile: need whole warps and at most 128 threads");
    if (pair != 0 && pair != 1) return ens_fail(e, EWPT_ERR_ARG, "pair must be 0 or 1");
    if (pair)
        for (const auto& p : e->mp)
            if (p.nx % 2) return ens_fail(e, EWPT_ERR_ARG, "paired sites need an even nx in every member");
    e->tile = Tiling{bx, by, 2, pair};  // at most 168 registers: 3 blocks of 128 threads per SM
    for (ewpt_ctx* c : e->mem) c->tile = e->tile;
    e->dirty = true;
    return EWPT_OK;
}

int ewpt_ensemble_set_member_tiling(ewpt_ens* e, int32_t m, int32_t bx, int32_t by, int32_t reg, int32_t pair) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (pair != 0 && pair != 1) return ens_fail(e, EWPT_ERR_ARG, "pair must be 0 or 1 for ensemble members");
    ewpt_ctx* c = e->mem[m];
    rc = ewpt_set_tiling(c, bx, by, reg, pair);  // the single-lattice checks
    if (rc) return ens_fail(e, rc, c->err.c_str());
    e->dirty = true;
    return EWPT_OK;
}

int ewpt_ensemble_step(ewpt_ens* e, int32_t nsteps) {
    if (!e) return ewpt_fail(nullptr, EWPT_ERR_ARG, "ensemble is NULL");
    if (nsteps < 0) return ens_fail(e, EWPT_ERR_ARG, "nsteps < 0");
    cudaSetDevice(e->device);
    if (nsteps > 0 && e->dirty) {
        int rc = ens_capture(e);
        if (rc) return rc;
    }
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

int64_t ewpt_ensemble_sites(const ewpt_ens* e) { return e ? e->sites : -1; }

int ewpt_ensemble_init_bubbles(ewpt_ens* e, int32_t m, int32_t nb, const double* bubbles, int32_t profile, double p0,
                               double p1) {
    int rc = ens_member_check(e, m);
    if (rc) return rc;
    if (nb < 0 || (nb > 0 && !bubbles)) return ens_fail(e, EWPT_ERR_ARG, "bubble list");
    if (profile != EWPT_BUBBLE_REFERENCE && profile != EWPT_BUBBLE_TANH) return ens_fail(e, EWPT_ERR_ARG, "profile");
    cudaSetDevice(e->device);
    const ewpt_params& p = e->mp[m];
    ewpt_ctx* c = e->mem[m];
    std::string err;
    rc = ewpt_launch_bubbles(c->g, p.dx, nb, bubbles, profile, profile == EWPT_BUBBLE_REFERENCE ? p.mH : p0, p1, p.vev,
                             nullptr, c->y32.hi, c->y32.lo, c->lay, e->st, &err);
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
    rc = ens_view(e, m, &v, false);
    if (rc) return rc;
    std::string err;
    rc = ewpt_thermal_fill(v->g, v->p, T, mH, mW, seed, v->y, e->st, &err, gauss_iters);
    if (rc) return ens_fail(e, rc, ("init_thermal: " + err).c_str());
    ewpt_ctx* c = e->mem[m];
    cudaError_t ce = launch_fp32_split(c->g, c->lay, v->y, c->y32, e->st);
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
