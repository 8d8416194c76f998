/*
 * hyperelastic.h -- C ABI of libhyperelastic_cuda.so, the GB300 (sm_103a)
 * explicit first-order finite-volume step of BlackSiberian/HyperelasticSolver.
 *
 * The reference is a set of pure Julia functions called per cell from a
 * threaded driver loop. This library replaces that hot path with whole-array,
 * device-resident calls. Every entry point below names the reference interface
 * it stands in for (file:line in the reference project).
 *
 * Conventions
 *  - Status: every function returns int, HYP_OK (0) on success; no exception
 *    or longjmp crosses the ABI. hyp_last_error() gives a message for a context.
 *  - Arrays are structure-of-arrays, double precision, in HOST memory unless a
 *    name says otherwise: x[k * n + i] is component k of cell/item i (a Julia
 *    Matrix{Float64}(n, k) has exactly this layout).
 *  - 3x3 tensors are column-major 9-vectors, as the reference's reshape(x,(3,3)).
 *  - Single-phase state (14 per cell): rho, rho*u(3), rho*E, rho*A(9) -- the
 *    reference's per-phase 15-vector (HyperelasticityMPh.jl:80-84) with the
 *    volume fraction alpha == 1 dropped. Two-phase state (30 per cell): the
 *    reference's [alpha, alpha*rho, alpha*rho*u(3), alpha*rho*E, alpha*rho*A(9)]
 *    for phase 1 then phase 2.
 *  - A context owns one CUDA stream and its device buffers; it is not
 *    thread-safe, the library is (one context per host thread).
 */
#ifndef HYPERELASTIC_H
#define HYPERELASTIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define HYP_OK 0
#define HYP_ERR_INVALID 1     /* null pointer, bad size, bad enum                          */
#define HYP_ERR_CUDA 2        /* CUDA runtime error (message in hyp_last_error)            */
#define HYP_ERR_NEG_DET 3     /* det(rho A) <= 0 in a cell: the reference's sqrt DomainError
                                 (HyperelasticityMPh.jl:114)                                 */
#define HYP_ERR_NONFINITE 4   /* non-finite state, wave speed or time step                 */
#define HYP_ERR_TIMEOUT 5     /* a bounded device-side wait gave up                         */
#define HYP_ERR_UNSUPPORTED 6 /* option combination not implemented                         */
#define HYP_ERR_NO_DEVICE 7   /* no CUDA device                                             */

enum { HYP_MODEL_SINGLE = 1, HYP_MODEL_MULTI = 2 };
/* numerical flux: Rusanov (local max speed per face, main.jl:45-48 with NumFluxes.lxf),
   Lax-Friedrichs (lambda = dx/dt, main.jl:223, 30-41), path-conservative HLL
   (NumFluxes.jl:70-132, main.jl:225) */
enum { HYP_FLUX_RUSANOV = 0, HYP_FLUX_LXF = 1, HYP_FLUX_HLL = 2 };
/* boundary: end cells frozen as main.jl:219-220, or zero-gradient (transmissive) ghosts */
enum { HYP_BC_FROZEN = 0, HYP_BC_TRANSMISSIVE = 1 };
/* arithmetic: plain FP64, or FP32 fluxes with a compensated hi/lo FP32 state */
enum { HYP_PREC_FP64 = 0, HYP_PREC_MIXED = 1 };
/* two-phase relaxation after each step (hyp_set_relaxation): none (the reference's
   model), instantaneous pressure relaxation, or velocity then pressure relaxation
   (mechanical equilibrium) */
enum { HYP_RELAX_NONE = 0, HYP_RELAX_PRESSURE = 1, HYP_RELAX_MECHANICAL = 2 };

/* Barton2009 primary parameters (EquationsOfState.jl:71-116); b0sq and k0 are derived.
   Defaults of the reference constructor: 8.93, 4.6, 3.9e-4, 300, 2.1, 1, 3, 2. */
typedef struct {
  double rho0, c0, cv, t0, b0, alpha, beta, gamma;
} hyp_barton2009;

typedef struct {
  int64_t n_cells;     /* nx (main.jl:143)                                      */
  int model;           /* HYP_MODEL_*                                           */
  int flux;            /* HYP_FLUX_*                                            */
  int bc;              /* HYP_BC_*                                              */
  int precision;       /* HYP_PREC_*                                            */
  double x_length;     /* X, domain [0, X] (main.jl:140); dx = X / nx           */
  double cfl;          /* main.jl:144                                           */
  hyp_barton2009 eos[2]; /* eos[1] is used by the two-phase model only (main.jl:134) */
} hyp_config;

typedef struct hyp_ctx hyp_ctx;

/* ---- solver context: the time loop of main.jl:202-241 -------------------- */

/* Create a context on the current CUDA device; allocates the state buffers. */
int hyp_create(const hyp_config* cfg, hyp_ctx** out);
int hyp_destroy(hyp_ctx* ctx);
/* Message of the last failure on this context (never NULL). */
const char* hyp_last_error(const hyp_ctx* ctx);
/* Cell index recorded with the last HYP_ERR_NEG_DET / HYP_ERR_NONFINITE, or -1. */
int64_t hyp_error_cell(const hyp_ctx* ctx);

/* Copy a conservative state in (host SoA [n_vars][n_cells]); resets t to t0.
   Replaces main.jl's Q0 = initial_condition(...) (main.jl:99-106, 178-179). */
int hyp_upload(hyp_ctx* ctx, const double* Q, int64_t n_cells, int n_vars, double t0);
/* Copy the current conservative state out (host SoA). */
int hyp_download(hyp_ctx* ctx, double* Q, int64_t n_cells, int n_vars);

/* Advance while steps < max_steps (max_steps <= 0: no limit) and t < t_end
   (t_end = +inf: no limit), exactly as `while t < T` of main.jl:202-241:
   per step, wave speeds of every cell (:204-211), dt = cfl*dx/max lambda
   (:212), t += dt (:214), update of the interior cells with frozen ends
   (:218-226). Reports the steps taken and the new time. */
int hyp_step(hyp_ctx* ctx, int max_steps, double t_end, int* steps_done, double* t_out);
/* Replace the Barton2009 parameters (EquationsOfState.jl:71-116) of one phase of a
   context: phase 0, or 1 for a two-phase context. The state and time are kept; the
   next step uses the new EOS (the reference passes eos to every call, main.jl:134,
   so a driver may change it between steps). A recorded adjoint run is discarded. */
int hyp_set_eos(hyp_ctx* ctx, int phase, const hyp_barton2009* eos);
/* Two-phase contexts: relaxation applied to every cell after each step; off
   (HYP_RELAX_NONE) by default. The reference has no relaxation terms (its two-phase
   model, HyperelasticityMPh.jl, ends at the non-conservative interface terms); this
   is an extension with no reference to match. HYP_RELAX_PRESSURE: instantaneous
   pressure relaxation (Saurel, Petitpas & Berry 2009) with hyperelastic phases as
   Favrie, Gavrilyuk & Saurel 2009 treat them: volume fractions move until both
   phases' mean-stress pressures agree, each phase's internal energy follows
   de = -p* dv and its distortion changes in its volumetric part only; each phase's
   mass and momentum and the mixture's total energy are conserved.
   HYP_RELAX_MECHANICAL first relaxes the velocities: both phases take the mixture
   velocity, each phase's total energy changing by m u* . (u* - u) so that the
   mixture's momentum and energy are kept; pressure relaxation alone lets the phases'
   velocities drift apart at a diffuse interface (on the smoothed-interface workload
   of 2^22 cells the minority phase's density then collapsed within 100 steps).
   Cells with a phase below 1e-5 are left as they are; with frozen ends the end cells
   too. Mixed contexts relax in FP64. A cell that does not converge is left
   unrelaxed and the step returns HYP_ERR_NONFINITE with its index. */
int hyp_set_relaxation(hyp_ctx* ctx, int mode);
/* The same relaxation (mode HYP_RELAX_PRESSURE or HYP_RELAX_MECHANICAL) of n two-phase
   cells (function level).  Q, Q_out: [30][n]; a cell that does not converge comes
   back as NaN. */
int hyp_eval_relax(const hyp_config* cfg, int mode, const double* Q, double* Q_out, int64_t n);
/* hyp_step (max_steps >= 1) that also returns the time after every step taken,
   t_hist[0 .. *steps_done - 1] (host, max_steps entries): the Step / t / dt line
   main.jl:229-237 logs each step, read back once at the end rather than with a
   host round trip per step. dt of step j is t_hist[j] - t_hist[j - 1] (the time
   before the call for j = 0). The steps run hyp_step's kernels, launched one by
   one (not from its CUDA graphs), each followed by a one-thread copy of its time,
   so state and times agree bitwise with hyp_step at a few microseconds more per
   step. */
int hyp_step_times(hyp_ctx* ctx, int max_steps, double t_end, int* steps_done, double* t_out, double* t_hist);

/* max_i lambda_i of the current state, lambda_i = max |get_eigvals(Q_i)|
   (main.jl:204-211; HyperelasticityMPh.jl:252-266). */
int hyp_max_wavespeed(hyp_ctx* ctx, double* out);

/* Current time and step count of the context. */
int hyp_get_time(const hyp_ctx* ctx, double* t, int64_t* steps);

/* Device timing of the last hyp_step: total elapsed ms, and when profiling is
   on, each step split in two, summed over the steps with their counts: first the
   per-cell flux/wave-speed kernel (two phases: with the face kernel, except in the
   mixed HLL step, whose faces run in one kernel with the update), then the rest. */
int hyp_set_profiling(hyp_ctx* ctx, int on);
int hyp_last_timing(const hyp_ctx* ctx, double* ms_total, double* ms_cell_kernel, int* cell_launches,
                    double* ms_update_kernel, int* update_launches);

/* Single-phase FP64 steps on caller-owned device buffers, allocating nothing.
   No counterpart in the reference: it serves callers that cannot allocate device
   memory where they step the solver (device memory owned by another allocator,
   or a latency-critical loop that must not call cudaMalloc). d_Q_in / d_Q_out are
   device SoA states [14][n_cells] (may be the same buffer); cfg must be
   single-phase, FP64, Rusanov or LxF, with cfg->n_cells == n_cells. The step's
   scratch is one fixed static device array sized for at most 65,536 cells
   (13,631,552 bytes = 13.0 MiB per GPU that loads the library, held until exit);
   larger n_cells is rejected with HYP_ERR_INVALID. The call synchronises `stream`
   (it reads the step's status back), so it cannot be made inside a stream capture
   or a CUDA graph. Calls share the array, so calls that overlap on the GPU race. Runs
   n_steps CFL steps from time t0 on `stream` (a cudaStream_t, NULL = the legacy
   default stream: pass the stream that produced d_Q_in, or synchronise first),
   waits for that stream to finish, and reports the new time; on HYP_ERR_NEG_DET /
   HYP_ERR_NONFINITE the first failing cell is stored in *err_cell. A CUDA launch
   error left pending by the caller's earlier work is cleared on entry, not
   reported. */
int hyp_step_noalloc_f64(const hyp_config* cfg, const double* d_Q_in, double* d_Q_out, int64_t n_cells, int n_steps,
                         double t0, void* stream, double* t_out, int64_t* err_cell);

/* Kernel family of a mixed-precision context.
   Single-phase: HYP_MIXED_TILE, one block per tile loading its own cells (the
   default, the fastest on GB300); HYP_MIXED_TMA, a persistent kernel whose tiles are prefetched by TMA;
   HYP_MIXED_PAIR, one block per two tiles, each thread stepping one cell of each
   in the lanes of packed FP32 pairs (f32x2 instructions). All three run the same
   tile arithmetic; the pair kernel's fused multiply-adds are written out, so its
   results differ from the others' in the last bits (within the mixed step's own
   error).
   Two-phase: HYP_MIXED_TILE, the face kernels with both phases in scalar FP32 and
   a separate update kernel; HYP_MIXED_PAIR (the default), the face kernels with the
   two phases as the lanes of packed FP32 pairs, computing the update in the same
   kernel. HYP_MIXED_TMA is single-phase only.
   Returns HYP_ERR_UNSUPPORTED for FP64 contexts, an unknown kind, or TMA where it
   is not available; the CUDA graphs of the previous kernel are dropped. */
enum { HYP_MIXED_TILE = 0, HYP_MIXED_TMA = 1, HYP_MIXED_PAIR = 2 };
int hyp_set_mixed_kernel(hyp_ctx* ctx, int kind);

/* Poll budget of the TMA kernel's device-side barrier waits (default 2^20). A wait
   that runs out records HYP_CELL_TIMEOUT, lets its in-flight copy land and ends the
   block, and the step returns HYP_ERR_TIMEOUT; the context stays usable (upload a
   state again). A budget of 0 makes every wait run out at once: the timeout path
   exercised without a fault. */
int hyp_set_wait_limit(hyp_ctx* ctx, int tries);

/* ---- domain decomposition: a context as one slab of a longer 1D domain ------ */
/* The reference advances one domain with a thread pool over its cells (main.jl:206,
   221). Split across processes (one GPU each), rank r's context holds the cells it
   updates plus a ghost cell at each inner end (its neighbour's boundary cell), and
   one step of main.jl:202-241 becomes: hyp_slab_local_max on every rank, a
   max-allreduce of those values (the caller's communicator), hyp_slab_step with the
   result, then the exchange of boundary cells (hyp_get_cells on the owner,
   hyp_set_cells into the neighbour's ghost). The max is exact and every face sees the
   cells it would see in one domain, so with the global dx the slabs step bitwise like
   the single-domain run. Single-phase contexts (Rusanov or LxF, FP64 or mixed). */
/* Make ctx a slab: dx of the global domain (X / global cells), whether its first and
   last cells are ghosts (held by the step; the global ends keep cfg->bc). hyp_step
   then refuses the context (a slab needs the global max). */
int hyp_set_slab(hyp_ctx* ctx, double dx, int left_ghost, int right_ghost);
/* Max wave speed over the cells the slab owns (ghosts excluded where their value is
   stale) of the current state; FP64 runs the step's cell pass to get it. */
int hyp_slab_local_max(hyp_ctx* ctx, double* lam);
/* One step with the global max wave speed: dt = cfl dx / lam_max (main.jl:212),
   t += dt, owned cells updated, ghosts held. Reports the new time. */
int hyp_slab_step(hyp_ctx* ctx, double lam_max, double* t_out);
/* Bytes per cell of a cell record: 112 (FP64: the 14 conservative values) or 128
   (mixed: 14 hi, 14 lo FP32 parts, the cell's FP32 wave speed and its 3 island
   outputs, so a ghost arrives with what its owner computed). */
int hyp_cell_record_size(const hyp_ctx* ctx, int* bytes);
/* Copy the records of cells [first, first + count) of the current state out to / in
   from rec, laid out [row][count] (rows of 8-byte doubles or 4-byte floats as above);
   rec may be host or device memory. */
int hyp_get_cells(hyp_ctx* ctx, int64_t first, int64_t count, void* rec);
int hyp_set_cells(hyp_ctx* ctx, int64_t first, int64_t count, const void* rec);

/* ---- batches of independent single-phase problems -------------------------- */
/* The reference advances one problem per main.jl run (main.jl:202-241). A batch
   advances n_problems independent problems of uneven size in lockstep, each with
   its own dx = X / N_p, CFL time step (main.jl:212) and time. Problem p owns cells
   [offsets[p], offsets[p+1]) of the SoA state [14][offsets[n_problems]]; cfg is
   single-phase (Rusanov or LxF, FP64 or mixed) with cfg->n_cells == offsets[n_problems]. */
typedef struct hyp_batch hyp_batch;
int hyp_batch_create(const hyp_config* cfg, const int64_t* offsets, int n_problems, hyp_batch** out);
int hyp_batch_destroy(hyp_batch* b);
const char* hyp_batch_last_error(const hyp_batch* b);
int hyp_batch_upload(hyp_batch* b, const double* Q, double t0);
int hyp_batch_download(hyp_batch* b, double* Q);
/* Every problem takes n_steps steps (one whose time reaches t_end stops there);
   the n_steps launches run as one CUDA graph. */
int hyp_batch_step(hyp_batch* b, int n_steps, double t_end);
/* Per-problem time and step count (arrays of n_problems). */
int hyp_batch_status(hyp_batch* b, double* t, int64_t* steps);
/* Device time of the last hyp_batch_step. */
int hyp_batch_last_ms(const hyp_batch* b, double* ms);
/* Mixed precision: time each tile-kernel variant for trial_steps steps on the
   batch's own state (restored afterwards) and keep the fastest; ms_per_step
   receives HYP_BATCH_NUM_VARIANTS timings. Every variant steps 254-cell tiles with
   256-thread blocks: 0, 1: a persistent grid (one wave striding over the tiles) at
   4 / 3 resident blocks per SM; 2 (the default): one block per tile. */
#define HYP_BATCH_NUM_VARIANTS 3
int hyp_batch_autotune(hyp_batch* b, int trial_steps, int* chosen, double* ms_per_step);
int hyp_batch_set_variant(hyp_batch* b, int variant);

/* ---- adjoint of the single-phase FP64 Rusanov run -------------------------- */
/* The reference has no derivative code; these entry points are what a Julia
   ChainRulesCore.rrule around a run of hyp_step binds: the forward pass records,
   the pullback calls hyp_adjoint. They cover single-phase FP64 contexts with the
   Rusanov flux (main.jl:45-48, 225), frozen or transmissive ends.

   hyp_adjoint_record: n_steps steps from the current state, as hyp_step with no
   t_end, keeping the state every ckpt_every steps (the first one included). */
int hyp_adjoint_record(hyp_ctx* ctx, int n_steps, int ckpt_every, double* t_out);
/* Reverse pass through the recorded run, which must end at the context's current
   state: from dL/dQ of the final state (host [14][n]) it returns dL/dQ of the
   recorded run's initial state (host [14][n], may be NULL) and dL_deos[2] =
   (dL/d b0sq, dL/d k0), the Barton2009 shear and bulk moduli of
   EquationsOfState.jl:111-112, each with the other held fixed. Segments between
   checkpoints are recomputed with the forward step kernels (bit-identical), then
   stepped backwards. dt = cfl dx / max lambda is differentiated through the
   arg-max cell (the smallest index among equal maxima). */
int hyp_adjoint(hyp_ctx* ctx, const double* dL_dQ_final, double* dL_dQ0, double* dL_deos);
/* Device times (ms) of the last hyp_adjoint_record and of the recompute and
   adjoint phases of the last hyp_adjoint. */
int hyp_adjoint_timing(const hyp_ctx* ctx, double* ms_record, double* ms_recompute, double* ms_adjoint);
/* Density misfit of the current state, L = 1/2 sum_i (rho_i - target_i)^2 with
   rho_i = sqrt(det(rho A)_i / rho0) (HyperelasticityMPh.jl:114; the density
   main.jl:71 writes), and dL/dQ (host [14][n], may be NULL). */
int hyp_density_misfit(hyp_ctx* ctx, const double* rho_target, double* loss, double* dL_dQ);

/* ---- snapshots and restart (main.jl:62-95, 108, 174-198, 233-237) ---------- */
/* cons2prim of the current state (per phase [alpha, rho, u(3), S, A(9)]) to host
   P [cols][n], cols = 15 (single phase, alpha = 1) or 30. */
int hyp_snapshot(hyp_ctx* ctx, double* P);
/* The reference's save_data file of the current state: tab-separated header
   a1 r1 u11 u21 u31 S1 F111 ... F331 [a2 ... F332], one row per cell, shortest
   round-trip numbers in Julia's layout. */
int hyp_save_snapshot(hyp_ctx* ctx, const char* path);
/* read_data + prim2cons (main.jl:79-95, 186-191): the file's prims become the
   current state at time t0 (the reference restarts at t = step * dt). */
int hyp_load_snapshot(hyp_ctx* ctx, const char* path, double t0);
/* The main.jl time loop with logging: saves dir/sol_%06i.csv for the current
   state (step number first_step) and after every step whose number is a multiple
   of log_freq, until t >= t_end or max_steps steps (either may be unbounded,
   not both); a run that reaches t_end also saves dir/result.csv (main.jl:242-244).
   Copies and file writing overlap the following steps. */
int hyp_run_logged(hyp_ctx* ctx, double t_end, int max_steps, int log_freq, const char* dir, int64_t first_step,
                   int* steps_done, double* t_out);

/* ---- initial conditions built on the device --------------------------------- */
/* HyperelasticityMPh.initial_states(eos, testcase) (HyperelasticityMPh.jl:275-426):
   the conservative left and right 30-vectors of test case 1-7 or 10 for the two
   phases of cfg (two-phase config). */
int hyp_initial_states(const hyp_config* cfg, int testcase, double* Ql, double* Qr);
/* initial_condition(Ql, Qr, nx) (main.jl:99-106) generated on the device as the
   current state at t = 0: cells (i - 1) < nx/2 (1-based) take Ql (nvar values). */
int hyp_init_riemann(hyp_ctx* ctx, const double* Ql, const double* Qr);
/* initial_condition_tanh(eos, Ql, Qr, nx, eps) (main.jl:110-123), two phases: per
   cell the primitive state of its side with alpha1 = 0.1 (tanh(4 (x - 1/2)/eps) + 1)
   + 0.4 and alpha2 = 1 - alpha1, x = (i - 1/2)/nx. */
int hyp_init_tanh(hyp_ctx* ctx, const double* Ql, const double* Qr, double eps);

/* Measured rates of this GPU for the roofline denominators the step needs (no
   counterpart in the reference, which publishes no hardware figures): out[0..5] =
   FP64 FMA TFLOP/s, FP32 FMA TFLOP/s, packed f32x2 FMA TFLOP/s, host-to-device GB/s,
   device-to-host GB/s, and GB/s each way with both directions at once (page-locked
   buffers of `bytes`); each the best of `reps`. */
int hyp_measure_peaks(int reps, int64_t bytes, double* out);

/* The single-phase mixed step's memory traffic (32 FP32 rows per cell read, the
   owned cells' rows written: 256 B per cell) for n_cells cells without the physics,
   in a row-major block (out[0], GB/s) and in the tile-major block the step uses
   (out[1], GB/s); each the best of `reps`. */
int hyp_measure_layouts(int reps, int64_t n_cells, double* out);

/* Page-locked host memory for staging states (fast, asynchronous-capable copies). */
int hyp_host_alloc(int64_t bytes, void** out);
int hyp_host_free(void* p);

/* ---- function-level evaluators (host arrays, n items, SoA) --------------- */
/* Each runs the same device code as the step on n independent inputs.       */

/* Strains.finger (Strains.jl:26-32): G = inv(A A^T).  A, G: [9][n] */
int hyp_eval_finger(const double* A, double* G, int64_t n);
/* Strains.invariants (Strains.jl:46-52): (tr G, (tr^2 G - tr G^2)/2, det G).  out: [3][n] */
int hyp_eval_invariants(const double* G, double* out, int64_t n);
/* EquationsOfState.energy(eos, S, G) (EquationsOfState.jl:118-137).  S, e: [n]; G: [9][n] */
int hyp_eval_energy(const hyp_barton2009* eos, const double* S, const double* G, double* e, int64_t n);
/* EquationsOfState.entropy(eos, e, G) (EquationsOfState.jl:139-156). */
int hyp_eval_entropy(const hyp_barton2009* eos, const double* e, const double* G, double* S, int64_t n);
/* EquationsOfState.stress(eos, ent, F) (EquationsOfState.jl:179-190).  sigma: [9][n] */
int hyp_eval_stress(const hyp_barton2009* eos, const double* S, const double* F, double* sigma, int64_t n);
/* EquationsOfState.acoustic(eos, ent, F, [1,0,0]) (EquationsOfState.jl:223-246).  [9][n] */
int hyp_eval_acoustic(const hyp_barton2009* eos, const double* S, const double* F, double* ac, int64_t n);
/* EquationsOfState.acoustic(eos, ent, F, n) (EquationsOfState.jl:223-246) for a direction
   n per item (dir: [3][n], not necessarily unit length, used as given).  ac: [9][n] */
int hyp_eval_acoustic_dir(const hyp_barton2009* eos, const double* S, const double* F, const double* dir, double* ac,
                          int64_t n);
/* EquationsOfState.stress(eos, den, e_int, F) (EquationsOfState.jl:162-176): the entropy
   from e_int (entropy(eos, e_int, finger(F)), clamped as :152-154), then
   -2 den G dE/dG with den as given.  den, e_int: [n]; F, sigma: [9][n] */
int hyp_eval_stress_den(const hyp_barton2009* eos, const double* den, const double* e_int, const double* F,
                        double* sigma, int64_t n);
/* EquationsOfState.acoustic(eos, P, n) (EquationsOfState.jl:192-221): P = one phase's
   primitive 15-vector [alpha, rho, u(3), S, A(9)]; e_int = energy(eos, S, finger(A)),
   then the Jacobian over F of stress(eos, alpha*rho, e_int, F) at F = A (the entropy
   following F at fixed e_int), divided by alpha*rho.  P: [15][n]; dir: [3][n]; ac: [9][n] */
int hyp_eval_acoustic_prim(const hyp_barton2009* eos, const double* P, const double* dir, double* ac, int64_t n);

/* Hank2016 (EquationsOfState.jl:305-366), which the reference defines at function
   level only (its time step uses Barton2009). Defaults: rho0 2.7, mu 26e9, gamma 3.4,
   pres_inf 21.5e9, a 0.5. */
typedef struct {
  double rho0, mu, gamma, pres_inf, a;
} hyp_hank2016;
/* energy(eos, den, pres, G) (:321-336).  den, pres, e: [n]; G: [9][n] */
int hyp_eval_hank2016_energy(const hyp_hank2016* eos, const double* den, const double* pres, const double* G,
                             double* e, int64_t n);
/* pressure(eos, den, e_int, i) (:338-352).  inv: [3][n] invariants of G */
int hyp_eval_hank2016_pressure(const hyp_hank2016* eos, const double* den, const double* e_int, const double* inv,
                               double* pres, int64_t n);
/* stress(eos, den, pressure, distortion) (:354-361): -2 den G dE/dG with G = finger(inv(F)).  F, sigma: [9][n] */
int hyp_eval_hank2016_stress(const hyp_hank2016* eos, const double* den, const double* pres, const double* F,
                             double* sigma, int64_t n);

/* Model-level functions; cfg selects model and EOS (n_cells etc. ignored).
   cons2prim / prim2cons (HyperelasticityMPh.jl:99-133, 63-90): per phase
   [alpha, rho_true, u(3), S, A(9)] (single phase: alpha dropped). [nvar][n] */
int hyp_eval_cons2prim(const hyp_config* cfg, const double* Q, double* P, int64_t n);
int hyp_eval_prim2cons(const hyp_config* cfg, const double* P, double* Q, int64_t n);
/* Pullback of single-phase prim2cons: Pbar = (dQ/dP)^T Qbar per item ([14][n]),
   eos_bar[2] = sum over items of (dL/d b0sq, dL/d k0). */
int hyp_eval_prim2cons_vjp(const hyp_config* cfg, const double* P, const double* Qbar, double* Pbar, double* eos_bar,
                           int64_t n);
/* flux_mph / flux (HyperelasticityMPh.jl:140-175).  [nvar][n] */
int hyp_eval_flux(const hyp_config* cfg, const double* Q, double* F, int64_t n);
/* get_eigvals (HyperelasticityMPh.jl:252-266) with n = e1: per phase
   u1 + c_k (k = 1..3) then u1 - c_k, c_k = sqrt|mu_k|, mu_k the eigenvalues of the
   acoustic tensor in the order Julia's eigvals returns them (HyperelasticityMPh.jl:263):
   ascending real part (LinearAlgebra's default sort).  out: [6*phases][n] */
int hyp_eval_eigvals(const hyp_config* cfg, const double* Q, double* out, int64_t n);
/* get_eigvals(eos, Q, n) for a direction per item: u.n +- sqrt|mu_k| of
   acoustic(eos, S, A, n), same order.  dir: [3][n]; out: [6*phases][n] */
int hyp_eval_eigvals_dir(const hyp_config* cfg, const double* Q, const double* dir, double* out, int64_t n);
/* NumFluxes.lxf(eos, Q_l, Q_r, lambda) (NumFluxes.jl:25-60): conservative part
   and the path-conservative D-, D+.  Ql, Qr, cons, dm, dp: [nvar][n]; lambda: [n] */
int hyp_eval_lxf(const hyp_config* cfg, const double* Ql, const double* Qr, const double* lambda, double* cons,
                 double* dm, double* dp, int64_t n);

/* Two-phase non-conservative matrix B(Q) (HyperelasticityMPh.noncons_flux,
   HyperelasticityMPh.jl:178-250). Only columns 1 and 16 of the 30x30 B are
   non-zero; bcol[r] = B[r,1] for r < 15 and B[r,16] for r >= 15.  [30][n] */
int hyp_eval_noncons(const hyp_config* cfg, const double* Q, double* bcol, int64_t n);
/* Two-phase path-conservative HLL fluctuations (NumFluxes.hll, NumFluxes.jl:70-132)
   with the wave speeds of Q_l and Q_r as main.jl:225 passes them; the conservative
   part the reference returns is zeros(30).  Ql, Qr, dm, dp: [30][n] */
int hyp_eval_hll(const hyp_config* cfg, const double* Ql, const double* Qr, double* dm, double* dp, int64_t n);
/* NumFluxes.hll(eos, Q_l, Q_r, eigvals) (NumFluxes.jl:70-132) with the caller's
   speeds, as the reference takes them: s_l = min(0, min speed of the face midpoint,
   minimum(eig_l)), s_r = max(0, max speed of the midpoint, maximum(eig_r))
   (NumFluxes.jl:90-91).  eig_l, eig_r: [12][n] (eigvals[1], eigvals[2]) */
int hyp_eval_hll_eigvals(const hyp_config* cfg, const double* Ql, const double* Qr, const double* eig_l,
                         const double* eig_r, double* dm, double* dp, int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* HYPERELASTIC_H */
