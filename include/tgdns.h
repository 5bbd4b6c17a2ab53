/*
 * tgdns.h - C ABI of the GB300-native Taylor-Green pseudo-spectral time step.
 *
 * This is the drop-in boundary for the hot path of mahanr/jax_tg_project
 * (Fourier pseudo-spectral RK4 on the periodic box [0, 2pi)^3 with the 2/3
 * dealias rule and a Leray projection, hydro and MHD).  The reference has no
 * FFI: its boundary is the Python function API of jax/taylor_green_jax.py and
 * of the CuPy shims cuda/taylor_green_cuda.py and cuda/taylor_green_mhd.py.
 * Each entry point below names the reference function it replaces.  The
 * Python package jax_tg_project_gb300 binds these with ctypes.
 *
 * Conventions
 *  - Every function returns TG_OK (0) or a TG_E_* code and never exits;
 *    tg_last_error() returns the message of the calling thread's last failure.
 *  - All buffer pointers are DEVICE pointers owned by the caller.  The plan
 *    owns its scratch buffers and tables.  Work is asynchronous on the plan's
 *    stream (tg_set_stream; default: the legacy default stream).
 *  - Spectral state ("state"): Fourier coefficients c_k (u(x) = sum c_k e^{ik.x})
 *    of the dealiased half spectrum, complex (float2 or double2) laid out
 *    [batch][F][M][M][Hz] with F = 3 (u) or 6 (u, b), M = 2K+1 kept modes per
 *    full axis ordered k = 0..K, -K..-1, kz = 0..K stored in rows of Hz >= K+1
 *    (entries kz > K are padding and never read).  K is the 2/3 cutoff of
 *    jax/taylor_green_jax.py:62-67 (n/3 for every supported n).
 *  - Physical fields: real (float or double) [batch][F][n][n][n], index
 *    (component, x, y, z) with z fastest, as the reference's (3, N, N, N)
 *    "ij" meshgrid arrays (jax/taylor_green_jax.py:70-79).
 *  - One plan per stream; a plan is not re-entrant.
 */
#ifndef TGDNS_H
#define TGDNS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tg_plan tg_plan;

enum {
  TG_OK = 0,
  TG_E_INVALID = 1,     /* bad argument (message says which) */
  TG_E_UNSUPPORTED = 2, /* grid size / precision combination not built */
  TG_E_CUDA = 3,        /* CUDA runtime error (message has the CUDA text) */
  TG_E_NOMEM = 4,       /* device allocation failed */
  TG_E_NONFINITE = 5    /* a diagnostic came out NaN/Inf */
};

enum { TG_PHYS_HYDRO = 0, TG_PHYS_MHD = 1 };
enum { TG_PREC_F32 = 0, TG_PREC_F64 = 1 };
enum {
  TG_FLAG_EXPLICIT_VISC = 1, /* classical RK4 with explicit viscosity (the reference's
                                scheme) instead of the integrating-factor RK4 */
  TG_FLAG_LORENTZ_REF = 2,   /* momentum RHS uses -(j x b) as the reference CuPy MHD
                                code does (cuda/taylor_green_mhd/operators.py:88-92)
                                instead of the physical +(j x b) */
  TG_FLAG_AUTOTUNE = 4       /* tg_plan_create times the pass variants (register-resident
                                or shared-memory x and z passes) on this plan's shape and
                                batch, then the y-pass configurations (radix plan and kz
                                columns per CTA), and keeps the fastest (tg_pass_variant,
                                tg_y_config).  TG_PASS_VARIANT / TG_Y_CONF in the environment
                                force a choice; with TG_AUTOTUNE_CACHE naming a file, choices
                                are read from and appended to it.  No reference counterpart */
};
enum {
  TG_IC_TAYLOR_GREEN = 0,     /* u = (sin x cos y cos z, -cos x sin y cos z, 0); b = 0 */
  TG_IC_MHD_REFERENCE = 1,    /* TG u and b = b_amp * (u_x, u_y, 0)
                                 (cuda/taylor_green_mhd/initial_conditions.py:9-21) */
  TG_IC_MHD_EQUAL_ENERGY = 2, /* TG u and b = (cos x sin y sin z, sin x cos y sin z,
                                 -2 sin x sin y cos z) / sqrt(3): E_m = E_k = 1/8 */
  TG_IC_ZERO = 3
};
enum { TG_ABSMAX_VELOCITY = 0, TG_ABSMAX_DIVERGENCE = 1 };
enum { TG_DERIVED_VORTICITY = 0, TG_DERIVED_DIVERGENCE = 1 };

/* Number of doubles per diagnostics record, and their order. */
#define TG_DIAG_WIDTH 8
enum {
  TG_D_KINETIC = 0,     /* 0.5 <|u|^2>            jax/taylor_green_jax.py:199-201 */
  TG_D_ENSTROPHY = 1,   /* 0.5 <|curl u|^2>       jax/taylor_green_jax.py:112-115 */
  TG_D_DISSIPATION = 2, /* nu sum |k|^2 |u_k|^2    jax/taylor_green_jax.py:118-128 */
  TG_D_MAGNETIC = 3,    /* 0.5 <|b|^2>            cuda/taylor_green_mhd/diagnostics.py:24 */
  TG_D_CROSS_HELICITY = 4, /* <u . b>             cuda/taylor_green_mhd/diagnostics.py:25-29 */
  TG_D_TOTAL = 5,       /* E_k + E_m */
  TG_D_DIVU_MAX = 6,    /* max |div u| in physical space  jax/taylor_green_jax.py:90-96 */
  TG_D_DIVB_MAX = 7     /* max |div b|            cuda/taylor_green_mhd/diagnostics.py:32-33 */
};

typedef struct tg_desc {
  int n;         /* grid points per axis: 8,12,16,24,32,48,64,96,128,256,512 (f32);
                    8,16,32,64,96,128,256 (f64) */
  int batch;     /* independent runs of this size advanced together (>= 1) */
  int physics;   /* TG_PHYS_* */
  int precision; /* TG_PREC_* */
  int flags;     /* TG_FLAG_* */
  int cutoff;    /* kept |k| per axis; <= 0 selects the reference 2/3 rule */
} tg_desc;

/* One device per process: kernels' shared-memory attributes are set once per process, on
 * the device current at their first launch; drive several GPUs as one process each. */
/* Create / destroy a plan (scratch buffers, twiddle tables, CUDA graphs).
 * Replaces the set-up of SpectralGrid (cuda/taylor_green_cuda/grid.py:5-13),
 * make_wavenumbers / make_dealias_mask (jax/taylor_green_jax.py:55-67) and the
 * cufftPlan3d calls of cuda/taylor_green_cuda.cu:102. */
int tg_plan_create(tg_plan** plan, const tg_desc* desc);
int tg_plan_destroy(tg_plan* plan);
int tg_set_stream(tg_plan* plan, void* cuda_stream);

/* Layout query: dims = {batch, F, M, M, Hz, K, n}; returns the number of complex
 * elements of a state buffer (0 on error). */
int64_t tg_state_layout(const tg_plan* plan, int dims[7]);
/* Bytes of device scratch the plan holds. */
int64_t tg_plan_scratch_bytes(const tg_plan* plan);

/* Per-run coefficients (count == batch, or 1 to broadcast).  Used by tg_step /
 * tg_run when they are called with dt <= 0. lorentz_sign is set from the plan flags. */
int tg_set_run_params(tg_plan* plan, const double* nu, const double* eta, const double* dt, int count);

/* Initial condition into a state buffer.  Replaces initial_taylor_green
 * (jax/taylor_green_jax.py:70-79), initial_taylor_green_spectral
 * (cuda/taylor_green_cuda.py:21-27) and initial_taylor_green_mhd[_spectral]
 * (cuda/taylor_green_mhd.py:22-31).  If pert_amp > 0 a seeded divergence-free
 * perturbation with spectrum E(k) ~ k^4 exp(-2 k^2/k0^2) and per-component rms
 * pert_amp is added to u; run r uses seed + r.  Synchronises the stream. */
int tg_initial_condition(tg_plan* plan, int kind, uint64_t seed, double pert_amp, double k0,
                         double b_amp, void* state);

/* Physical field -> dealiased state (fftn + mask, cuda/taylor_green_cuda/grid.py:31-34). */
int tg_forward(tg_plan* plan, const void* phys, void* state);
/* State -> physical field (ifftn(...).real, cuda/taylor_green_cuda/grid.py:36-37). */
int tg_inverse(tg_plan* plan, const void* state, void* phys);

/* Spectral RHS of the dealiased state: -P[mask F(u.grad u)] - nu k^2 u (hydro,
 * jax/taylor_green_jax.py:158-185 in spectral form, cuda/taylor_green_cuda/operators.py:24-48)
 * or the MHD pair (cuda/taylor_green_mhd/operators.py:70-107).  nu < 0 uses the
 * per-run table. */
int tg_rhs(tg_plan* plan, const void* state, double nu, double eta, void* rhs_out);

/* Advance the state nsteps RK4 steps in place (jax/taylor_green_jax.py:188-196,
 * cuda/taylor_green_cuda/integrator.py:7-12, cuda/taylor_green_mhd/integrator.py:14-32).
 * dt <= 0 uses the per-run table set by tg_set_run_params. */
int tg_step(tg_plan* plan, void* state, double dt, double nu, double eta, int nsteps);

/* The run loop (jax/taylor_green_jax.py:266-275, cuda/taylor_green_mhd/simulation.py:59-68):
 * records diagnostics of the initial state, then after every save_every steps
 * and after the last step.  series (device) receives [records][batch][TG_DIAG_WIDTH]
 * doubles with records = 1 + nsteps/save_every + (nsteps % save_every != 0).
 * Synchronises at the end and returns TG_E_NONFINITE if any recorded value is NaN/Inf
 * (the series is still written; the message names the first bad record). */
int tg_run(tg_plan* plan, void* state, double dt, double nu, double eta, int nsteps,
           int save_every, double* series);

/* One diagnostics record per run into out (device, [batch][TG_DIAG_WIDTH]): per-mode
 * terms in the state's precision, deterministic FP64 sums; the divergence maxima come
 * from a physical-space transform.  Replaces kinetic_energy / enstrophy / viscous_dissipation /
 * spectral_divergence (jax/taylor_green_jax.py:90-128,199-201) and
 * MhdDiagnostics.record (cuda/taylor_green_mhd/diagnostics.py:20-49). */
int tg_diagnostics(tg_plan* plan, const void* state, double nu, double eta, double* out);

/* max over physical points of |field| (TG_ABSMAX_VELOCITY: per component of u
 * [and b]; TG_ABSMAX_DIVERGENCE: div u [, div b]) into out (device, [batch][F or F/3]).
 * Used for validate_timestep's max_velocity (jax/taylor_green_jax.py:257). */
int tg_field_absmax(tg_plan* plan, const void* state, int which, double* out);

/* Physical-space derived fields of a state into phys (device, real):
 * TG_DERIVED_VORTICITY: curl u [, curl b] ([batch][F][n][n][n]); replaces vorticity
 * (jax/taylor_green_jax.py:99-109) and spectral_curl (cuda/taylor_green_mhd/operators.py:24-25).
 * TG_DERIVED_DIVERGENCE: div u [, div b] ([batch][F/3][n][n][n]); replaces
 * spectral_divergence (jax/taylor_green_jax.py:90-96) and divergence_from_hat
 * (cuda/taylor_green_mhd/operators.py:50-51). */
int tg_derived(tg_plan* plan, const void* state, int which, void* phys);

/* Conversion between the state and the full complex fftn layout of the CuPy
 * solvers ([batch][F][n][n][n] complex, unnormalised, dealiased modes only):
 * the spectral arrays of cuda/taylor_green_cuda.py:21-46 and cuda/taylor_green_mhd.py:28-59.
 * tg_from_full_spectrum keeps only the kept modes with kz >= 0 (the input is
 * taken to be the spectrum of a real field). */
int tg_to_full_spectrum(tg_plan* plan, const void* state, void* full);
int tg_from_full_spectrum(tg_plan* plan, const void* full, void* state);

/* 0.5 <|u|^2> [and 0.5 <|b|^2>] of a physical field in FP64 ([batch][F/3] doubles):
 * kinetic_energy (jax/taylor_green_jax.py:199-201) / magnetic_energy
 * (cuda/taylor_green_mhd.py:62-69) evaluated on the grid values as given. */
int tg_physical_energy(tg_plan* plan, const void* phys, double* out);

/* Per-pass timing: runs nsteps RK4 steps eagerly (no graph) with a CUDA event
 * pair around every kernel launch on the plan's stream, then writes, per pass
 * kind (slot = internal pass op: 0/1 x-stage hydro/MHD, 2/3 x-load, 4/5 x-forward,
 * 6 y-inverse, 7 y-forward, 8/9 z-product hydro/MHD, 10 z-C2R, 11 z-R2C), the mean
 * launch duration in ms and the launch count.  The reference has no profiler; its
 * only timing is wall-clock around the loop (jax/taylor_green_jax.py:264,277). */
#define TG_PROF_SLOTS 12
int tg_profile_passes(tg_plan* plan, void* state, double dt, double nu, double eta, int nsteps,
                      double ms[TG_PROF_SLOTS], int64_t count[TG_PROF_SLOTS]);

/* Pass variant in use: bit 0 set = shared-memory z passes, bit 1 set = shared-memory x
 * passes, bit 2 set (without bit 1) = the hydro x stage with the column's spectral values
 * stashed in shared memory between its phases (n = 64 ... 256) (0: register-resident passes
 * where they are built).  Chosen by TG_FLAG_AUTOTUNE, else 0 (or the TG_PASS_VARIANT
 * environment variable).  No reference counterpart. */
int tg_pass_variant(const tg_plan* plan);

/* y-pass configuration in use (0 = the default radix plan and tile width); *count (if not
 * null) receives the number of configurations built for this size and precision.  Chosen by
 * TG_FLAG_AUTOTUNE, else 0 (or the TG_Y_CONF environment variable).  No reference
 * counterpart. */
int tg_y_config(const tg_plan* plan, int* count);

/* Kernels launched by the last tg_step / tg_run call (for launch accounting). */
int64_t tg_last_launch_count(const tg_plan* plan);

/* Discrete adjoint of nsteps integrating-factor RK4 steps (hydro, batch 1):
 * loss = enstrophy of the final state (jax/taylor_green_jax.py:112-115 applied at
 * t_final).  Writes loss (device double), grad_state = dloss/dstate0 (device, state
 * layout; the gradient for the inner product sum_half w Re(a conj b), w = 1 at
 * kz = 0 and 2 otherwise) and grad_nu = dloss/dnu (device double).
 * checkpoint_every > 0: states are checkpointed every checkpoint_every steps (0: every
 * ceil(sqrt(nsteps)) steps) and each segment is recomputed on the way back.  With the
 * stage-tape kernels (FP32 plans with register passes, n = 16 ... 256) the recompute of a
 * segment records its step tape (the step's state and stage nonlinear terms, 4 states per
 * step) in pinned host memory and the backward sweep reads it; the checkpoints and the
 * adjoint state are held in pinned host memory meanwhile (the plan keeps that memory for
 * later calls), so the device holds only the plan, the working state and 8 tape states.
 * Other plans recompute each step's stage terms on the device.
 * TG_ADJ_HOST_TAPE: one forward sweep records the tape of every step in pinned host
 * memory and nothing is recomputed (with the stage-tape kernels; else, or if the host
 * memory cannot be pinned, the sqrt(nsteps) checkpointing runs instead).
 * The reference has no adjoint; its autodiff counterpart is jax.grad through
 * jax/taylor_green_jax.py:188-196.  Allocates its device work buffers for the call and
 * synchronises the stream. */
#define TG_ADJ_HOST_TAPE (-1)

/* Phases of the plan's last stage-tape tg_adjoint call, in ms of device time (CUDA events on
 * the plan's stream): ms[0] the forward run (with the tape recorded, or keeping the segment
 * checkpoints) and the loss, ms[1] the tape recording sweeps of the segments (0 for the
 * whole-run tape), ms[2] the backward sweeps.  No reference counterpart. */
int tg_adjoint_profile(const tg_plan* plan, double ms[3]);

/* Free the pinned host memory a TG_ADJ_HOST_TAPE adjoint keeps in the plan for later calls
 * (the plan stays usable; the next tape adjoint pins it again).  No reference counterpart. */
int tg_release_host_tape(tg_plan* plan);
int tg_adjoint(tg_plan* plan, const void* state0, double dt, double nu, int nsteps, int checkpoint_every,
               void* grad_state, double* grad_nu, double* loss);

/* Shell-summed energy spectrum E(k) = 0.5 sum_{round(|k|) = k} |u_k|^2 (full-spectrum sum)
 * for k = 0 .. tg_spectrum_bins(plan)-1, per run into out (device doubles,
 * [batch][bins] for hydro, [batch][2][bins] (kinetic, magnetic) for MHD).  Not in the
 * reference (a natural extension of its diagnostics); deterministic summation order. */
int tg_spectrum_bins(const tg_plan* plan);
int tg_energy_spectrum(tg_plan* plan, const void* state, double* out);

/* Allocation-free diagnostics.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory when they need the energies (a
 * framework that owns all device memory and forbids cudaMalloc inside its
 * operators, a fixed-footprint real-time loop) and therefore cannot create a
 * plan.  Computes records 0-5 of tg_diagnostics (E_k, enstrophy, nu*sum k^2|u|^2,
 * E_m, H_c, E_k+E_m) of a state laid out as a plan with the default 2/3 cutoff
 * would lay it out (n, batch, physics, precision as in tg_desc) into out
 * ([batch][TG_DIAG_WIDTH] doubles, device); slots 6-7 (divergence maxima) are
 * not computed and are set to -1.  n must be a size tg_plan_create builds for the
 * precision (else TG_E_UNSUPPORTED); nu >= 0 is used as given (there is no plan
 * whose nu a negative value could select: TG_E_INVALID).  Its only scratch is a
 * file-scope device array of TG_NOALLOC_MAX_RUNS*96*5 doubles (240 KiB) that every
 * GPU loading the library holds until the process exits; batch >
 * TG_NOALLOC_MAX_RUNS is rejected with TG_E_INVALID.  The first call on each device
 * (more exactly: in each CUDA context, so again after a device reset) looks up the
 * array's device address (cudaGetSymbolAddress) with that device current: make that
 * first call before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race and must be ordered by the caller.  Calls no
 * cudaMalloc/cudaFree and no allocating library routine.  eta is unused (kept for
 * symmetry with tg_diagnostics).  Asynchronous on stream. */
#define TG_NOALLOC_MAX_RUNS 64
int tg_diagnostics_noalloc(const void* state, int n, int batch, int physics, int precision, double nu,
                           double eta, double* out, void* stream);

const char* tg_last_error(void);
int tg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TGDNS_H */
