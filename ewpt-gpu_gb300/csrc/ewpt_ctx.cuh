// ewpt_ctx.cuh -- the context object behind the opaque ewpt_ctx handle.
#pragma once
#include <cstdarg>
#include <string>

#include "ewpt_internal.cuh"

struct ewpt_ctx {
    ewpt_params p{};
    Grid g{};
    cudaStream_t st = nullptr;
    int64_t it = 0;  // RK4 iterations done (the reference's loop counter)
    bool view = false;  // state buffer only (an ensemble member's FP64 view): no stepping
    // z-slab of a larger lattice (slab.cu): g.nz interior planes starting at
    // global plane z0 of nz_global, g.zg ghost planes per z face
    bool slab = false;
    int z0 = 0, nz_global = 0;
    Tiling tile = kDefaultTiling;  // stage-kernel launch shape
    // FP64 form: state y, accumulator yn, stage inputs xa/xb, each [36][S]
    double* y = nullptr;
    double* yn = nullptr;
    double* xa = nullptr;
    double* xb = nullptr;
    // DF64 form: [12][S] float pairs passing the Higgs currents between the
    // launches of a split stage (stage_dd.cu)
    double* ddcur = nullptr;
    // FP32 form: compensated state, weighted rate sum, float stage inputs
    Fp32State y32{nullptr, nullptr};  // all five FP32 buffers: [36][lay.P]
    Layout lay{};
    void* tma = nullptr;  // TMA stage-kernel state (stage_tma.cu), made by the first TMA tiling
    int64_t wait_polls = -1;  // limit of the TMA kernels' mbarrier waits in polls (< 0: default)
    Fp32Work w32{nullptr, nullptr, nullptr};
    bool fp32_comp = false;  // FP32 form: compensated gauge stencils (ewpt_set_fp32_compensated)
    // side streams and events of the host <-> device state copies: the
    // chunked copies (api.cu copy_runs) use io_st[0..2] and io_ev[0..3], the
    // overlapped host-to-host steps (ewpt_step_host) all of them
    cudaStream_t io_st[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t io_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // [36][S] doubles: FP64 view of an FP32 state (diagnostics, get/set)
    double* scratch64 = nullptr;
    // diagnostics / spectra scratch (diag.cu, spectrum.cu)
    double* red = nullptr;      // per-block partial sums
    int red_blocks = 0;
    double* dres = nullptr;     // device result row
    double* field3 = nullptr;   // [3 or 4][S] real fields for the FFT
    void* fft_out = nullptr;    // complex half-spectrum buffers
    int fft_plan = 0;           // cufftHandle
    int fft_ready = 0;
    double* shell = nullptr;    // per-shell accumulators
    std::string err;
};

int ewpt_fail(ewpt_ctx* ctx, int code, const char* fmt, ...);
int ewpt_cuda_check(ewpt_ctx* ctx, cudaError_t e, const char* what);
int ewpt_validate_params(const ewpt_params* p, ewpt_ctx* ctx);
// FP64 context holding only the state buffer, for diagnostics and spectra of
// a state that lives elsewhere (ensemble members).
extern "C" int ewpt_create_view(const ewpt_params* p, ewpt_ctx** out);
// FP64 view of the current state: c->y for FP64 contexts; for FP32 contexts
// the state joined into c->scratch64.
int ewpt_state64(ewpt_ctx* c, const double** out);
int ewpt_ensure_scratch64(ewpt_ctx* c);
// FP64 [36][S] buffer to write a whole state into (c->y, or the FP32 form's
// scratch64), and the conversion of a state written there into the
// context's form (FP32 split with ghost faces, DF64 pairs), on c->st.
extern "C" int ewpt_staging64(ewpt_ctx* c, double** out, bool in);
extern "C" cudaError_t ewpt_commit_staged(ewpt_ctx* c, const double* staged);
// Interior of a slab context <-> a packed [36][nx ny nz] buffer (slab.cu).
cudaError_t ewpt_slab_copy(ewpt_ctx* c, double* packed, bool to_dev, int32_t on_device);
// Thermal IC (thermal.cu) into an FP64 [36][S] device state y, synchronous
// on st; ewpt_check_thermal validates T and the masses.
int ewpt_thermal_fill(const Grid& g, const ewpt_params& p, double T, double mH, double mW, uint64_t seed,
                      double* y, cudaStream_t st, std::string* err, int gauss_iters);
int ewpt_check_thermal(double T, double mH, double mW);
void ewpt_release_aux(ewpt_ctx* c);
// Bubble IC kernel (init.cu) on an FP64 state (y) or an FP32 hi/lo state.
// TMA-staged FP32 stage kernels (stage_tma.cu).
bool tma_tiling_fits(const Grid& g, int by, int bz);
int ewpt_tma_prepare(ewpt_ctx* c, int by, int bz);
void ewpt_tma_release(ewpt_ctx* c);
void ewpt_tma_set_spin(ewpt_ctx* c);
int ewpt_tma_check(ewpt_ctx* c);
cudaError_t launch_step_fp32_tma(ewpt_ctx* c, double Jex, double gam);
// For the FP32 form, L is the hi/lo buffers' layout (ghost images of hi written).
int ewpt_launch_bubbles(const Grid& g, double dx, int nb, const double* bubbles, int profile, double p0, double p1,
                        double p2, double* y, float* hi, float* lo, const Layout& L, cudaStream_t st,
                        std::string* err);
