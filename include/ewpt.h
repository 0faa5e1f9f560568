/*
 * ewpt.h -- C ABI of libewpt, the GB300 (sm_103a) implementation of the
 * real-time RK4 lattice evolution of the electroweak bosonic sector of
 * Teerthal/EWPT-GPU.
 *
 * Plain C types only (no CUDA or torch types): a Julia `ccall`, Python
 * `ctypes` or C caller binds these directly.  Every entry point returns an
 * int status (EWPT_OK = 0); the message of the last failure is returned by
 * ewpt_last_error().
 *
 * Array order.  The state is 36 real arrays of nx*ny*nz doubles, each in
 * Julia column-major order (linear index i + nx*(j + ny*k), x fastest), i.e.
 * exactly the memory of a CuArray{Float64,3}.  Order of the 36 arrays:
 *    0- 3  phi_1..phi_4                  (Higgs doublet, 4 real components)
 *    4-12  W_1_2 W_1_3 W_1_4  W_2_2 .. W_3_4   (W^a_i, a = 1..3, i = x,y,z)
 *   13-15  Y_2 Y_3 Y_4                   (hypercharge)
 *   16-18  Gamma_1..Gamma_3, 19 Sigma    (Gauss-constraint auxiliaries)
 *   20-23  dphi_a_dt, 24-32 dW_a_i_dt, 33-35 dY_i_dt   (momenta)
 * The rates ("k" and "kt" arrays of rk4_step!) use the same order: rate a
 * is d/dt of array a.
 *
 * Threading: one context is bound to one CUDA stream and must be used from
 * one host thread at a time; distinct contexts are independent.
 */
#ifndef EWPT_H
#define EWPT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EWPT_NARR 36
#define EWPT_NDIAG 20

enum ewpt_status {
    EWPT_OK = 0,
    EWPT_ERR_ARG = 1,       /* invalid argument (dims, null pointer, non-finite parameter) */
    EWPT_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    EWPT_ERR_CUFFT = 3,     /* a cuFFT call failed */
    EWPT_ERR_OOM = 4,       /* device allocation failed */
    EWPT_ERR_NONFINITE = 5, /* the state holds NaN/Inf */
    EWPT_ERR_TIMEOUT = 6,   /* a bounded device-side wait ran out */
    EWPT_ERR_STATE = 7      /* call not valid in the context's current state */
};

enum ewpt_precision {
    EWPT_FP64 = 0, /* stencils, fluxes, state and reductions in FP64 */
    EWPT_FP32 = 1, /* FP32 stencils and fluxes; compensated FP32 hi/lo RK4 state; FP64 reductions */
    EWPT_DF64 = 2  /* the FP64 form evaluated in double-float (float hi + lo) arithmetic on the
                      FP32 pipes: ~2^-47 per operation, FP64 reductions */
};

/* Parameter set.  Mirrors gpu-kernels-rk4/parameters.jl:1-98 (couplings,
 * lattice, dt = dx/ARG5, damping gamma_inp, beta_W/beta_Y, mH, t_sat) plus
 * the run() switch thermal_init (main_rk4.jl:7082) that enables the
 * J_ext/damp schedule of main_rk4.jl:5154-5172. */
typedef struct ewpt_params {
    int32_t nx, ny, nz;   /* lattice sites per axis, each >= 7 (parameters.jl:14) */
    int32_t precision;    /* enum ewpt_precision */
    double dx, dt;        /* parameters.jl:22-23 */
    double gw, gy, gp2;   /* parameters.jl:16-19 */
    double lambda, vev;   /* parameters.jl:20-21 */
    double theta_w;       /* Weinberg angle used by the B field, parameters.jl:17,26 */
    double beta_w, beta_y;/* CP-odd couplings, parameters.jl:34-35 */
    double gamma_inp;     /* damping after t_sat, parameters.jl:29 */
    double mH, t_sat;     /* J_ext/damp schedule, parameters.jl:24,40 */
    int32_t thermal_init; /* 1: apply J_ext/damp schedule (main_rk4.jl:5154-5172) */
    int32_t device;       /* CUDA device ordinal */
    int32_t stencil_order;/* central-difference order of every stencil: 6 (default; 0 means 6) or
                             2, 8, 10, 12 -- the modules of diff_scheme.jl:370-1438 that the
                             driver selects with `using` (main_rk4.jl:33-35).  Orders other than 6
                             need the FP64 form; every axis needs >= order + 1 sites. */
} ewpt_params;

typedef struct ewpt_ctx ewpt_ctx;

/* Fills p with the reference's defaults (parameters.jl) for an n^3 lattice:
 * gw = 0.65, gy = gw*tan(asin(sqrt(0.22))), gp2 = 0.99, lambda = 0.129,
 * vev = 1, dx = 0.25, dt = dx/10, mH = 2*sqrt(lambda)*vev, t_sat = 2. */
int ewpt_params_default(ewpt_params* p, int32_t n);

/* Allocates the device state of one lattice (replaces the CuArray
 * allocations of main_rk4.jl:5178-5304).  State starts at zero. */
int ewpt_create(const ewpt_params* p, ewpt_ctx** out);
int ewpt_destroy(ewpt_ctx* ctx);

/* Message of the last failure on ctx (ctx may be NULL: last failure of any
 * call that had no context).  Never NULL. */
const char* ewpt_last_error(const ewpt_ctx* ctx);

/* Copy the 36 state arrays in (set) or out (get).  arrays[a] points to
 * nx*ny*nz doubles on the host (on_device = 0) or on the context's device
 * (on_device = 1).  Replaces copyto!(CuArray, Array) / Array(CuArray). */
int ewpt_set_state(ewpt_ctx* ctx, const double* const arrays[EWPT_NARR], int32_t on_device);
int ewpt_get_state(ewpt_ctx* ctx, double* const arrays[EWPT_NARR], int32_t on_device);
/* Same with one packed buffer of 36*nx*ny*nz doubles (array-major). */
int ewpt_set_state_packed(ewpt_ctx* ctx, const double* buf, int32_t on_device);
int ewpt_get_state_packed(ewpt_ctx* ctx, double* buf, int32_t on_device);

/* nsteps classical RK4 steps (main_rk4.jl:6146-6437), asynchronous on the
 * context's stream.  Iteration it (1-based, counted by the context) uses
 * Jex = J_ext(it) and gamma = damp(it) (main_rk4.jl:5154-5172). */
int ewpt_step(ewpt_ctx* ctx, int32_t nsteps);
/* Same with explicit Jex and gamma for every step (counter still advances). */
int ewpt_step_explicit(ewpt_ctx* ctx, int32_t nsteps, double Jex, double gamma);
/* Host state in, nsteps RK4 steps, host state out, synchronous: the same
 * result as ewpt_set_state_packed(state_in, 0) + ewpt_step(nsteps) +
 * ewpt_get_state_packed(state_out, 0), bit for bit, and the same iteration
 * count and drive.  Both buffers hold 36*nx*ny*nz doubles (array-major) and
 * may be the same buffer; the new state also stays on the device.  FP64
 * contexts with 6th-order stencils, nz >= 16 and page-locked buffers
 * (cudaHostAlloc / cudaHostRegister) overlap the copies with the stencil
 * work: the upload goes in windows of z planes, stage 1 of the first step
 * starts on the planes that have arrived, and the planes that stage 4 of the
 * last step has finished go down while the rest is computed.  Other
 * contexts and pageable buffers take the three calls in turn.  Replaces the
 * copyto!(CuArray, Array) ... rk4 loop ... Array(CuArray) round trip of a
 * host-side driver (main_rk4.jl:5174-5304, 6146-6437). */
int ewpt_step_host(ewpt_ctx* ctx, const double* state_in, double* state_out, int32_t nsteps);
/* Iterations done so far (the `it` of the reference loop). */
int64_t ewpt_iteration(const ewpt_ctx* ctx);
/* Launch shape of the stage kernels.  pair = 0 or 1: blocks of bx*by
 * threads over x and y (whole warps, at most 128 threads), reg = register-
 * budget variant (0: registers at the compiler's choice; 1: <= 128
 * registers; 2: <= 168); pair = 1 (FP32 form, even nx): each thread evolves
 * two x-adjacent sites with packed FP32x2 arithmetic.  pair = 2 (FP32 form):
 * TMA-staged shared-memory tiles of bx x by x reg sites -- bx = 32, by = 4 or
 * 2, reg = 4 (the tile's z extent); needs nx % 32 == 0, ny % by == 0,
 * nz % 4 == 0 -- with the same arithmetic as pair = 1.  The result of a step
 * does not depend on bx, by or reg, and pair only changes FP32 rounding
 * (pair = 1 and 2 agree bit for bit); ewpt/autotune.py picks the fastest per
 * lattice size and precision.  Default 32x4, 0, 0. */
int ewpt_set_tiling(ewpt_ctx* ctx, int32_t bx, int32_t by, int32_t reg, int32_t pair);
int ewpt_get_tiling(const ewpt_ctx* ctx, int32_t* bx, int32_t* by, int32_t* reg, int32_t* pair);
/* FP32 form, compensated mode (on = 1; default 0): the gauge fields'
 * Laplacians and the Gauss auxiliaries' gradients are accumulated with
 * error-free transformations (a float pair, ~2^-44 of the terms) and the
 * combinations lap W^a_i - d_i Gamma^a and lap Y_i - d_i Sigma of the gauge
 * rates are formed before they are rounded to FP32.  For the longitudinal
 * gauge modes those two terms nearly cancel; rounded separately they leak
 * FP32 noise into the transverse (magnetic) modes, which sets the FP32
 * form's B-spectrum error.  Everything else stays FP32.  Needs a tiling
 * with pair = 1 (and keeps it: other tilings are refused while on); runs
 * with at most 168 registers whatever reg says.  No counterpart in the
 * reference. */
int ewpt_set_fp32_compensated(ewpt_ctx* ctx, int32_t on);
int32_t ewpt_get_fp32_compensated(const ewpt_ctx* ctx);
/* Limit of the device-side waits of the TMA-staged stage kernels (pair = 2),
 * in mbarrier polls; polls < 0 restores the default (2^22), 0 makes every
 * wait give up at once.  A wait that runs out ends the kernel's copies
 * safely, the step's results are invalid and the next ewpt_sync /
 * ewpt_get_state returns EWPT_ERR_TIMEOUT; the context stays usable (set
 * the state again).  For testing the bounded-wait path; no counterpart in
 * the reference. */
int ewpt_set_wait_limit(ewpt_ctx* ctx, int64_t polls);
/* Wait for all work queued on the context. */
int ewpt_sync(ewpt_ctx* ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void* ewpt_stream(ewpt_ctx* ctx);

/* Drop-in for one launch of rk4_step! (main_rk4.jl:52-661, launched at
 * :6155/:6226/:6298/:6370): reads the 20 fields + 16 momenta in[0..35]
 * (device pointers) and writes the 20 k + 16 kt rates out[0..35] (device
 * pointers), FP64, asynchronously on `stream` (a cudaStream_t or NULL).
 * in and out must not alias. */
int ewpt_rk4_rates(const ewpt_params* p, const double* const in[EWPT_NARR],
                   double* const out[EWPT_NARR], double Jex, double gamma, void* stream);

/* Snapshot diagnostics of the current state, FP64, one fused reduction
 * (replaces compute_PE!..compute_Az! + host sums, main_rk4.jl:6451-6805):
 *   out[0..6]  PE KE GE EEW MEW EEY MEY   (sum * dx^3; columns 1-7 of
 *              total_energies, main_rk4.jl:6790-6796)
 *   out[7]     0.5*sum(B^2)*dx^3          out[8]  0.5*sum(B_2^2)*dx^3
 *   out[9]     min |Phi|                  out[10] 0
 *   out[11]    mean |Phi|                 out[12] sum(B_2 . A)*dx^3
 *   out[13]    total energy = sum of out[0..6]  (main_rk4.jl:6921)
 *   out[14]    sqrt(sum_a sum G_a^2 dx^3), G_a = d_i E^a_i - rho^a (SU(2) Gauss law)
 *   out[15]    max |G_a|    out[16] sqrt(sum G_Y^2 dx^3)   out[17] max |G_Y|
 *   out[18]    sqrt(sum_a sum (Gamma_a - d_i W^a_i)^2 dx^3)
 *   out[19]    sqrt(sum (Sigma - d_i Y_i)^2 dx^3)
 * Synchronous.  Returns EWPT_ERR_NONFINITE (row still written) if any
 * column is NaN/Inf. */
int ewpt_diagnostics(ewpt_ctx* ctx, double out[EWPT_NDIAG]);

enum ewpt_field { EWPT_FIELD_B = 0, EWPT_FIELD_B2 = 1, EWPT_FIELD_HIGGS = 2, EWPT_FIELD_DENSITY = 3 };
enum ewpt_spec_mode { EWPT_SPEC_LOG = 0, EWPT_SPEC_UNIQUE = 1 };

/* Power spectrum of the current state (replaces fft(E_t) + convolve_1d,
 * main_rk4.jl:6580-6685 and spec_routines.jl:47-77).  P(n) = sum over the
 * components of |FFT(component)|^2 (unnormalised forward transform), FFT of
 *   EWPT_FIELD_B      B_x, B_y, B_z   (compute_Bx/By/Bz!, main_rk4.jl:2303-2822)
 *   EWPT_FIELD_B2     B_2 components  (compute_B_2_*!, main_rk4.jl:3718-4250)
 *   EWPT_FIELD_HIGGS  phi_1..phi_4 (DC mode removed).
 * mode EWPT_SPEC_LOG: nbins (<= 256) shells log-uniform in |n| over
 * [1, min(nx,ny,nz)/2], DC excluded; k[b] = geometric shell centre.
 * mode EWPT_SPEC_UNIQUE: one bin per distinct integer |n| in increasing
 * order, the first nbins of them (convolve_1d with
 * nbins = ewpt_kc_bin_nums(cut)); k[b] = |n|.
 * Writes sum, count (modes), mean = sum/count per bin; *nbins_out (may be
 * NULL) = bins written.  Synchronous. */
int ewpt_spectrum(ewpt_ctx* ctx, int32_t field, int32_t mode, int32_t nbins, double* k, double* sum,
                  double* count, double* mean, int32_t* nbins_out);

/* Per-site fields of the current state in FP64, one nx*ny*nz array per
 * component in the state's order (x fastest: a Julia Array{Float64,3}):
 *   EWPT_FIELD_B        3: B_x, B_y, B_z (the E_t of compute_Bx/By/Bz!)
 *   EWPT_FIELD_B2       3: B_2 components (compute_B_2_x/y/z!)
 *   EWPT_FIELD_HIGGS    4: phi_1..phi_4 as stored
 *   EWPT_FIELD_DENSITY  7: energy densities PE, KE, GE, EEW, MEW, EEY, MEY
 *                          (the E_t of compute_PE! .. compute_MEY!,
 *                          main_rk4.jl:1334-2301; sum * dx^3 = the energy)
 * The reference takes its y-slices (main_rk4.jl:6451-6560) and 3D B FFTs
 * (:6579-6868) from these arrays.  out holds ewpt_field_components(field)
 * * nx*ny*nz doubles, on the host (on_device = 0) or the device.  Synchronous
 * for host output. */
int32_t ewpt_field_components(int32_t field);
int ewpt_fields(ewpt_ctx* ctx, int32_t field, double* out, int32_t on_device);

/* Number of distinct |K| on a cx*cy*cz index lattice (Kc_bin_nums,
 * spec_routines.jl:32-43), -1 on bad input. */
int64_t ewpt_kc_bin_nums(int32_t cx, int32_t cy, int32_t cz);

enum ewpt_bubble_profile { EWPT_BUBBLE_REFERENCE = 0, EWPT_BUBBLE_TANH = 1 };

/* Bubble-nucleation initial condition on the device (replaces the per-bubble
 * initializer! launches, main_rk4.jl:4930-4946 and :5691-5697): phi_a =
 * sum_b d_ab * profile_b(x), every other array zero, iteration counter reset.
 * bubbles: nb rows of 7 doubles (centre cx, cy, cz, direction d1..d4).
 * EWPT_BUBBLE_REFERENCE: the reference's rmag(rb) profile with its
 *   sin-distance, centres in its 1-based site indices, mass = params.mH
 *   (p0, p1 unused).
 * EWPT_BUBBLE_TANH: vev * 0.5 * (1 - tanh((r - p0)/p1)), centres in physical
 *   units, r the minimum-image distance (p0 = radius, p1 = wall width). */
int ewpt_init_bubbles(ewpt_ctx* ctx, int32_t nb, const double* bubbles, int32_t profile, double p0, double p1);

/* Thermal initial condition generated on the device (replaces the thermal
 * branch of run(), main_rk4.jl:5348-5636, with thermal_initializer_phi! and
 * thermal_initializer_gauge!, :5029-5152): Bose-Einstein modes at
 * temperature T as real(bfft(amp (a + i b))), amp = sqrt(n(w) / (w V)),
 * a, b ~ N(0, sqrt 2); Higgs w^2 = k^2 + mH^2; W^a and Y with two transverse
 * polarisations and w^2 = k^2 + mW^2 (W) or k^2 (Y); Gamma^a and Sigma set
 * to the stencil divergence of W^a and Y; momenta zero.  Deviates are a
 * counter-based hash of (seed, field, mode): the state depends only on the
 * seed and the lattice.  Resets the iteration counter.  Synchronous. */
int ewpt_init_thermal(ewpt_ctx* ctx, double T, double mH, double mW, uint64_t seed);

/* The benchmark's precision-configuration IC: ewpt_init_thermal's fields
 * with thermal momenta as well (Higgs and gauge, amplitude sqrt(n(w) w / V),
 * the gauge momenta transverse, zero at k = 0), then gauss_iters iterations
 * of ewpt_gauss_project.  No counterpart in the reference, whose thermal
 * momenta are zero.  Resets the iteration counter.  Synchronous. */
int ewpt_init_thermal_gauss(ewpt_ctx* ctx, double T, double mH, double mW, uint64_t seed, int32_t gauss_iters);

/* Projects the current state's electric fields onto the discrete Gauss law
 * of the evolution (the gp2 parts of k_Gamma, k_Sigma, main_rk4.jl:603-655):
 * d_i E^a_i = rho^a, d_i E^Y_i = rho_Y with the 6th-order central difference.
 * Each of `iters` iterations first moves the Higgs momenta along the charge
 * generators so that the charges have no component in the zero and
 * staggered modes the divergence cannot produce, then subtracts grad chi
 * from each group's E, chi from a Fourier-space solve; the SU(2) charge
 * depends on E, so the residual falls by iterations.  The fields, Gamma and
 * Sigma are unchanged.  Any form (FP32/DF64 states are projected in FP64).
 * No counterpart in the reference.  Synchronous. */
int ewpt_gauss_project(ewpt_ctx* ctx, int32_t iters);

enum ewpt_thermal_flags {
    /* mode (i, j, k) of the spectrum array takes theta = 2 pi (index + 1) / N,
     * the reference's 1-based indexing (main_rk4.jl:5040-5046), instead of the
     * FFT frequency */
    EWPT_THERMAL_ONE_BASED_MODES = 1
};

/* The reference's thermal IC from the caller's random draws (replaces the
 * thermal branch of run(), main_rk4.jl:5348-5636, with its own deviate
 * arrays): thermal_initializer_gauge! and thermal_initializer_phi!
 * (:5029-5152) scale them and real(bfft(.)) makes the fields.  deviates
 * holds 44 arrays of nx*ny*nz doubles (x fastest), host (on_device = 0) or
 * device memory, in the order run() draws them: for W^1, W^2, W^3 and Y the
 * ten arrays r_1, r_2, r_3, r_1_i, r_2_i, r_3_i, x_1, x_2, x_3, x_4, then
 * phi_1_k .. phi_4_k.  Higgs w^2 = k^2 + mH^2 (the reference: mH^2 =
 * meff_sq, parameters.jl:37), W^a w^2 = k^2 + mW^2 (the reference: mW = 0),
 * Y massless; the gauge mode with k = 0 is left empty.  Gamma, Sigma and the
 * momenta are zero, as in run().  flags: enum ewpt_thermal_flags.  Resets
 * the iteration counter.  Synchronous. */
int ewpt_init_thermal_deviates(ewpt_ctx* ctx, double T, double mH, double mW, const double* deviates,
                               int32_t on_device, int32_t flags);

/* ---------------------------------------------------------------------
 * z-slab decomposition (replaces the MPI decomposition of
 * gpu-kernels-rk4/main_rk4_multiple.jl: update_halo! and boundary_x/y/z,
 * :69-212, host-staged MPI.Sendrecv! of 3-plane ghost layers after every
 * stage).  An nx x ny x nz lattice is cut along z into slabs; a slab keeps 3
 * ghost planes below and above its interior, filled from the neighbouring
 * slabs (periodic in z) before each RK4 stage.  FP64 form, 6th-order
 * stencils; a decomposed step gives the same bits as ewpt_step on the whole
 * lattice.
 *
 * One process, any number of slabs on one or several GPUs: */
typedef struct ewpt_slabs ewpt_slabs;
/* n slabs of nz_local[m] planes (NULL: an even split, the first nz % n
 * slabs one plane more; each >= 3), slab m on devices[m] (NULL: p->device).
 * p describes the whole lattice.  State starts at zero. */
int ewpt_slabs_create(const ewpt_params* p, int32_t n, const int32_t* nz_local, const int32_t* devices,
                      ewpt_slabs** out);
int ewpt_slabs_destroy(ewpt_slabs* slabs);
const char* ewpt_slabs_last_error(const ewpt_slabs* slabs);
int32_t ewpt_slabs_count(const ewpt_slabs* slabs);
/* the whole lattice's packed [36][nx*ny*nz] state, host or device memory
 * (set resets the iteration counter); synchronous */
int ewpt_slabs_set_state(ewpt_slabs* slabs, const double* packed, int32_t on_device);
int ewpt_slabs_get_state(ewpt_slabs* slabs, double* packed, int32_t on_device);
/* launch shape of every slab's stage kernels (ewpt_set_tiling, pair = 0) */
int ewpt_slabs_set_tiling(ewpt_slabs* slabs, int32_t bx, int32_t by, int32_t reg);
/* nsteps RK4 steps (the J_ext/damp schedule of ewpt_step, or explicit
 * values), asynchronous on the slabs' streams */
int ewpt_slabs_step(ewpt_slabs* slabs, int32_t nsteps);
int ewpt_slabs_step_explicit(ewpt_slabs* slabs, int32_t nsteps, double Jex, double gamma);
int ewpt_slabs_sync(ewpt_slabs* slabs);
void* ewpt_slabs_stream(ewpt_slabs* slabs, int32_t m);

/* One slab per process (a rank per GPU); the caller moves the packed faces.
 * A slab context of planes [z0, z0 + nz_local) of the lattice p (FP64,
 * 6th order, nz_local >= 3); its state I/O is ewpt_set/get_state_packed on
 * the packed [36][nx*ny*nz_local] interior.  One step is, for stage = 1..4:
 *   ewpt_slab_pack(ctx, stage, lo, hi)        the bottom / top 3 interior
 *       planes of the stage's input into lo / hi ([36][3*nx*ny] doubles each,
 *       device memory); send lo to the slab below, hi to the slab above;
 *   ewpt_slab_unpack(ctx, stage, below, above) the planes received from the
 *       slab below (its hi) and above (its lo) into the ghost planes;
 *   ewpt_slab_stage(ctx, stage, Jex, gamma)   the stage kernel.
 * All three are asynchronous on the context's stream (ewpt_stream). */
int ewpt_create_slab(const ewpt_params* p, int32_t z0, int32_t nz_local, ewpt_ctx** out);
int ewpt_slab_pack(ewpt_ctx* ctx, int32_t stage, double* lo, double* hi);
int ewpt_slab_unpack(ewpt_ctx* ctx, int32_t stage, const double* below, const double* above);
int ewpt_slab_stage(ewpt_ctx* ctx, int32_t stage, double Jex, double gamma);

/* ---------------------------------------------------------------------
 * Batched ensembles (no counterpart in the reference, which runs one
 * realization per process; each member here is an independent lattice with
 * its own size, couplings and dt, in the FP32 form).  Every member is an
 * FP32-form context evolved by the single-lattice stage kernels, so member m
 * evolves exactly like a single context with the same tiling.  One RK4 step
 * of all members is one CUDA graph with a branch per member; the branches
 * run concurrently on the GPU.  Members start at zero and carry per-member
 * Jex/gamma (default 0, see ewpt_ensemble_set_drive).
 */
typedef struct ewpt_ens ewpt_ens;
int ewpt_ensemble_create(int32_t n, const ewpt_params* members, ewpt_ens** out);
int ewpt_ensemble_destroy(ewpt_ens* ens);
const char* ewpt_ensemble_last_error(const ewpt_ens* ens);
int32_t ewpt_ensemble_size(const ewpt_ens* ens);
/* total lattice sites over all members */
int64_t ewpt_ensemble_sites(const ewpt_ens* ens);
/* packed [36][S_m] FP64 state of member m, host (on_device = 0) or device memory */
int ewpt_ensemble_set_state(ewpt_ens* ens, int32_t m, const double* packed, int32_t on_device);
int ewpt_ensemble_get_state(ewpt_ens* ens, int32_t m, double* packed, int32_t on_device);
/* ewpt_init_bubbles for member m */
int ewpt_ensemble_init_bubbles(ewpt_ens* ens, int32_t m, int32_t nb, const double* bubbles, int32_t profile,
                               double p0, double p1);
/* ewpt_init_thermal for member m (the same state as a single context of
 * the member's parameters and the same seed, split into the FP32 form) */
int ewpt_ensemble_init_thermal(ewpt_ens* ens, int32_t m, double T, double mH, double mW, uint64_t seed);
/* ewpt_init_thermal_gauss for member m */
int ewpt_ensemble_init_thermal_gauss(ewpt_ens* ens, int32_t m, double T, double mH, double mW, uint64_t seed,
                                     int32_t gauss_iters);
/* constant Jex and gamma of member m for the following steps */
int ewpt_ensemble_set_drive(ewpt_ens* ens, int32_t m, double Jex, double gamma);
/* launch shape of every member: bx*by threads (whole warps, <= 128), at
 * most 168 registers, pair = two x-adjacent sites per thread (every member
 * needs an even nx; default when possible).  Default 16x8 threads. */
int ewpt_ensemble_set_tiling(ewpt_ens* ens, int32_t bx, int32_t by, int32_t pair);
/* launch shape of member m alone, as ewpt_set_tiling (pair 0 or 1), e.g.
 * the shape a single lattice of that size runs fastest with */
int ewpt_ensemble_set_member_tiling(ewpt_ens* ens, int32_t m, int32_t bx, int32_t by, int32_t reg, int32_t pair);
/* nsteps RK4 steps of every member, asynchronous on the ensemble's stream */
int ewpt_ensemble_step(ewpt_ens* ens, int32_t nsteps);
int ewpt_ensemble_sync(ewpt_ens* ens);
void* ewpt_ensemble_stream(ewpt_ens* ens);
/* ewpt_diagnostics / ewpt_spectrum of member m */
int ewpt_ensemble_diagnostics(ewpt_ens* ens, int32_t m, double out[EWPT_NDIAG]);
int ewpt_ensemble_spectrum(ewpt_ens* ens, int32_t m, int32_t field, int32_t mode, int32_t nbins, double* k,
                           double* sum, double* count, double* mean, int32_t* nbins_out);

/* ---------------------------------------------------------------------
 * Learned surrogate (no counterpart in the reference): a 3-layer BF16 MLP
 * n_in -> width -> width -> n_out with GELU, FP32 accumulation on the tensor
 * cores, trained with AdamW on the GPU.  Parameters are FP32, flattened as
 * W1 [width][n_in], b1 [width], W2 [width][width], b2 [width],
 * W3 [n_out][width], b3 [n_out].  Inputs x [batch][n_in] and targets
 * y [batch][n_out] are FP32 host arrays; the loss is the mean squared error.
 */
typedef struct ewpt_mlp ewpt_mlp;
int ewpt_mlp_create(int32_t n_in, int32_t width, int32_t n_out, int32_t max_batch, int32_t device, ewpt_mlp** out);
int ewpt_mlp_destroy(ewpt_mlp* net);
const char* ewpt_mlp_last_error(const ewpt_mlp* net);
int64_t ewpt_mlp_num_params(const ewpt_mlp* net);
/* Limit of the tensor-core waits of the MLP GEMM in mbarrier polls (< 0: the
 * default 2^22; 0: every wait gives up at once, the call returns
 * EWPT_ERR_TIMEOUT and the net stays usable).  For testing. */
int ewpt_mlp_set_wait_limit(ewpt_mlp* net, int64_t polls);
/* set (resets the optimizer state) / get the FP32 parameters */
int ewpt_mlp_set_params(ewpt_mlp* net, const float* params);
int ewpt_mlp_get_params(ewpt_mlp* net, float* params);
/* y = net(x) */
int ewpt_mlp_forward(ewpt_mlp* net, const float* x, int32_t batch, float* y);
/* loss and d loss / d params (same layout as the parameters) at the current parameters */
int ewpt_mlp_gradients(ewpt_mlp* net, const float* x, const float* y, int32_t batch, float* grads, float* loss);
/* one AdamW step (beta1 0.9, beta2 0.999, eps 1e-8, decoupled weight decay); loss may be NULL */
int ewpt_mlp_train_step(ewpt_mlp* net, const float* x, const float* y, int32_t batch, float lr, float weight_decay,
                        float* loss);

/* Measured FP64 peak of `device` in FLOP/s (no counterpart in the
 * reference): a kernel of independent fused multiply-add chains on every SM,
 * timed with CUDA events (2 FLOPs per DFMA).  The denominator of the FP64
 * stage kernels' compute roofline, which are bound by the FP64 pipe.
 * *seconds (may be NULL) = the timed launch.  Synchronous; restores the
 * caller's current device. */
int ewpt_fp64_peak(int32_t device, double* flop_per_s, double* seconds);

/* Snapshot diagnostics (the same 20 columns as ewpt_diagnostics) of a
 * caller-owned FP64 state, without allocating any device memory.  No
 * counterpart in the reference: it is for callers that cannot let the
 * library call cudaMalloc, e.g. a process whose device memory belongs to
 * another allocator's pool, or a loop that must keep its device footprint
 * fixed.  `state` is a device pointer to 36*nx*ny*nz doubles in the order
 * above (packed, array-major); `out` is host memory; work is queued on
 * `stream` (a cudaStream_t or NULL) and the call waits for it.
 * Scratch lives in one fixed device array per GPU (1,048,832 bytes: 4096
 * partial rows of 32 doubles plus the final row, held until the process
 * exits), sized for at most 4096 x-y tiles of 32x4 sites
 * (ceil(nx/32)*ceil(ny/4) <= 4096, e.g. nx = ny = 512); larger lattices are
 * rejected with EWPT_ERR_ARG.  Each call looks up the array's device address
 * on p->device and restores the caller's current device before it returns.
 * The call copies the row into host memory and waits for its stream, so it
 * must not be called while that stream is being captured into a CUDA graph.
 * Calls share the array and each one overwrites it: calls whose work
 * overlaps on the GPU race and must be serialised by the caller. */
int ewpt_diagnostics_noalloc(const ewpt_params* p, const double* state, double out[EWPT_NDIAG], void* stream);

#ifdef __cplusplus
}
#endif
#endif /* EWPT_H */
