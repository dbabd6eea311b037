/*
 * gturbo.h -- C-ABI of the GB300-native time-stepping hot path of the Gturbo
 * 2D alpha-turbulence pseudo-spectral solver.
 *
 * Every entry point replaces one Fortran external of the reference (implicit
 * interface, arrays `present` on the device) and keeps its argument meaning:
 * the caller owns every field, passes DEVICE pointers to them (Fortran:
 * `!$acc host_data use_device(z,...)`), and the library owns only its tables
 * (wavenumbers, integrating factor, forcing list, twiddles) and, up to N = 2048,
 * one spectral scratch field for the field-split column passes.
 *
 * Memory layout of a field (identical to the reference), NX = n, NY = ny:
 *   spectral  complex(8) z(NX/2+1, NY) -> C: double z[NY][NX/2+1][2], kx fastest
 *   physical  real(8)    z(NX+2, NY)   -> C: double z[NY][NX+2], x fastest,
 *                                         2 padding doubles per row
 * Both views are the same NS = (NX+2)*NY doubles (src/modules.f90:4-9).
 *
 * Every function returns GT_OK (0) or a GT_ERR_* code; the message of the last
 * failure is returned by gt_last_error(h) (or gt_last_error(NULL) for a failed
 * gt_create). No C++ exception crosses this boundary.
 *
 * All work is enqueued on the handle's stream (gt_set_stream, default: the
 * legacy default stream) and is asynchronous unless stated otherwise.
 */
#ifndef GTURBO_H
#define GTURBO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GT_OK 0
#define GT_ERR_ARG 1      /* invalid argument or parameter                  */
#define GT_ERR_CUDA 2     /* a CUDA runtime call failed                      */
#define GT_ERR_NFORC 3    /* more forced modes than GT_NFORC ('NFORC too small !') */
#define GT_ERR_STATE 4    /* wrong call order / handle state                 */
#define GT_ERR_NOMEM 5    /* device or host allocation failed                */
#define GT_ERR_NONFINITE 6 /* a diagnostic reduction found NaN/Inf           */

/* Capacity of the forced-mode table: commforc NFORC (src/modules.f90:41). */
#define GT_NFORC 2048

/* Runtime parameters: the contents of params.dat (src/inieuler.f90:13-20)
 * plus the compile-time grid size NX, NY (src/modules.f90:4). */
typedef struct gt_params {
  int32_t n;        /* NX (row length, x fastest), a power of two in [16, 8192] */
  int32_t rko;      /* Runge-Kutta order, 2 or 4 (anything else -> 2, as inieuler.f90:241-243) */
  int32_t truncate; /* 1 = 2/3-rule dealiasing (trunc), 0 = none           */
  int32_t split;    /* -1 = derive as inieuler.f90:22-36; 0/1 = force     */
  double xlx, xly;  /* box lengths                                          */
  double nu, alpnu; /* hyperviscosity nu * k^(2 alpnu)                       */
  double mu, alpmu; /* friction mu * k^(2 alpmu)                            */
  double alpv;      /* alpha: psi_hat = -q_hat / |k|^alpha                  */
  double dt;        /* time step                                            */
  double rtrunc;    /* truncation radius as written in params.dat (unsquared) */
  double famp, k1f, k2f; /* forcing amplitude and shell k1f < |k| <= k2f     */
  int32_t ny;       /* NY (rows), a power of two in [16, 8192]; 0 = NX (square).
                     * A non-square grid has NX, NY >= 32. The reference declares NX
                     * and NY separately (modules.f90:4) but plans its transforms as
                     * NY x NY (main.f90:27,32); here every routine follows NX x NY.
                     * The ensemble, the tangent-linear model, the adjoint and
                     * gt_diag_static take square grids only.                     */
  int32_t ny_pad_;
} gt_params;

/* Derived quantities of a handle (read-only). */
typedef struct gt_info {
  int32_t n, nh;        /* NX and NX/2+1                                     */
  int32_t nbin;         /* NBIN = NX/2 (src/modules.f90:9)                   */
  int32_t rko, split, truncate;
  int32_t nf;           /* number of forced modes (iniforcing)              */
  int32_t ny;           /* NY                                                */
  int64_t field_doubles;/* NS = (NX+2)*NY                                    */
  double dkx, dky;
  double inpz, inpe;    /* mean enstrophy / energy input (iniforcing.f90:28-29) */
  double fkxsmax, fkysmax, rtrunc2;
} gt_info;

typedef struct gt_handle gt_handle;

/* ---- set-up ------------------------------------------------------------ */

/* Replaces the set-up half of inieuler (src/inieuler.f90:22-87): derives
 * split, dt2/dt3/dt6/sdt, runs defk (src/defk.f90:1-76) and iniforcing
 * (src/iniforcing.f90:1-80), and uploads the tables to the current device.
 * Returns GT_ERR_NFORC where the reference stops with 'NFORC too small !'. */
int gt_create(const gt_params* p, gt_handle** out);
int gt_destroy(gt_handle* h);
/* Stream for all later work; NULL = legacy default stream. */
int gt_set_stream(gt_handle* h, void* cuda_stream);
int gt_get_info(const gt_handle* h, gt_info* info);
/* Forced-mode table (iniforcing.f90: ikxf, ikyf; 0-based here). Host arrays
 * of capacity GT_NFORC. */
int gt_get_forcing_modes(const gt_handle* h, int32_t* ikxf, int32_t* ikyf, int32_t* nf);
/* Message of the last failure on h (h == NULL: last gt_create failure). */
const char* gt_last_error(const gt_handle* h);
/* Synchronise the handle's stream; returns any pending asynchronous error. */
int gt_sync(gt_handle* h);

/* ---- spectral transforms (src/fft_dir.f90, src/fft_inv.f90) ------------ */

/* In-place 2D real-to-complex FFT of the physical field followed by the
 * division by NY*NX of every value, padding included (src/fft_dir.f90:11-21). */
int gt_fft_dir(gt_handle* h, double* z);
/* In-place unnormalised 2D complex-to-real FFT (src/fft_inv.f90:11-13). The
 * imaginary parts of the kx=0 and kx=N/2 values after the y-transform are
 * taken as zero (Hermitian input); the 2 padding doubles per row are zeroed. */
int gt_fft_inv(gt_handle* h, double* z);
/* Field dump (src/main.f90:119-125 + src/write.f90:29-51 without the host-side
 * conversion): the physical field of the spectral field in `work` (destroyed,
 * normally a copy of z as the reference's znl = z) written to the DEVICE array
 * `out` as N*N real(4) values, x fastest: the record of fields/w.NNN.MMM. */
int gt_dump_real4(gt_handle* h, double* work, float* out);
/* Restart from a field dump (src/read.f90:3-27 readf, then src/main.f90:89-92):
 * the N*N real(4) physical values `in` (DEVICE array, x fastest: the record of
 * fields/w.NNN) are widened to real(8) with zero padding, transformed as
 * gt_fft_dir into the spectral field z, and truncated as gt_trunc when the
 * handle's truncate = 1. */
int gt_load_real4(gt_handle* h, const float* in, double* z);
/* 2/3-rule ellipse mask and zero mean, in place (src/trunc.f90:10-25). */
int gt_trunc(gt_handle* h, double* z);
/* Physical-space products u <- z*u, v <- z*v, padding zeroed (src/produ.f90:11-23). */
int gt_produ(gt_handle* h, const double* z, double* u, double* v);

/* ---- nonlinear term and time steppers ---------------------------------- */

/* Nonlinear term (src/nlt.f90:1-66): on return z holds N_hat = -i k.(u q)^,
 * truncated when truncate=1. z's input is destroyed as in the reference; u and
 * v are scratch fields of NS doubles each. */
int gt_nlt(gt_handle* h, double* z, double* u, double* v);
/* Lawson RK2 step (src/rkstep.f90:2-76); znl, u, v are scratch. */
int gt_step_rk2(gt_handle* h, double* z, double* znl, double* u, double* v);
/* Lawson RK4 step (src/rkstep.f90:82-131); znl, znew, u, v are scratch. */
int gt_step_rk4(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v);

/* ---- stochastic forcing (src/forcing.f90:1-51) -------------------------- */

/* Adds one white-in-time random-phase kick to the nf forced modes. *seed is
 * the caller's LCG state (host int32, as the Fortran `seed` variable):
 * it is read, and on return holds the state after nf draws. The phases are
 * bit-identical to the reference's serial rann() sequence. */
int gt_forcing(gt_handle* h, double* z, int32_t* seed);
/* The reference's rann (src/forcing.f90:40-51) on the host: advances *seed
 * once and returns the real(4) draw. Exported for drivers and tests. */
float gt_rann(int32_t* seed);
/* One step followed by one kick, the body of the reference's main loop on steps
 * without diagnostics (src/main.f90:100-106: step/step4, then forcing). The kick
 * is added in the final stage's store instead of a separate launch, as the
 * stage update's fused forcing injection. Results and *seed are bit-identical
 * to gt_step_rk2/gt_step_rk4 followed by gt_forcing. A handle whose forced
 * modes include a self-conjugate one (two kicks on one value, possible only
 * without truncation) runs the step and gt_forcing one after the other. */
int gt_step_rk2_forced(gt_handle* h, double* z, double* znl, double* u, double* v, int32_t* seed);
int gt_step_rk4_forced(gt_handle* h, double* z, double* znl, double* znew, double* u, double* v,
                       int32_t* seed);

/* Counter-based forcing, no counterpart in the reference (its LCG is serial):
 * the same kick as gt_forcing, with the phase of forced mode k at step `step`
 * equal to 2*pi*u, u = top 53 bits of Philox4x64-10(counter = (step, k, 0, 0),
 * key = (key, 0)) word 0. Independent streams per key; every mode is drawn in
 * parallel and the result does not depend on call order. */
int gt_forcing_philox(gt_handle* h, double* z, uint64_t key, uint64_t step);

/* ---- batched ensembles (no counterpart in the reference) ---------------- */

/* An ensemble advances nmembers independent fields in one launch per pass:
 * members may differ in grid size (powers of two in [128, 2048]), alpha,
 * dt, dissipation and forcing shell, but share the RK order. Member m has the
 * parameters members[m] and the Philox forcing stream keys[m]. One step of
 * every member is the RK step (gt_step_rk2/gt_step_rk4) followed by
 * gt_forcing_philox at the ensemble's step counter, which then advances. */
typedef struct gt_ens gt_ens;
int gt_ens_create(const gt_params* members, int32_t nmembers, const uint64_t* keys, gt_ens** out);
int gt_ens_destroy(gt_ens* e);
/* Stream the ensemble's work is ordered after / before (NULL = legacy default). */
int gt_ens_set_stream(gt_ens* e, void* cuda_stream);
/* Device fields of every member (host arrays of nmembers device pointers, each
 * field NS doubles of that member's size); znew may be NULL for RK2. */
int gt_ens_set_fields(gt_ens* e, double* const* z, double* const* znl, double* const* znew,
                      double* const* u, double* const* v);
/* Philox step counter of the next forcing (synchronous). */
int gt_ens_set_step(gt_ens* e, uint64_t step);
int gt_ens_get_step(gt_ens* e, uint64_t* step);
/* 1 (default): capture one ensemble step as a CUDA graph on first use and replay
 * it; 0: launch the kernels directly every step. */
int gt_ens_use_graph(gt_ens* e, int enable);
/* Advance every member by nsteps steps (asynchronous on the ensemble's stream). */
int gt_ens_step(gt_ens* e, int32_t nsteps);
/* Tile family of the ensemble's pass kernels: 16, 8 (default) or 4 complex values per thread,
 * 128, 256 or 512 threads per CTA; every CTA holds 2048 values of one member, so the families
 * differ only in the radix decomposition of the transforms (results agree to rounding). */
int gt_ens_set_tile(gt_ens* e, int32_t values_per_thread);
int gt_ens_get_tile(const gt_ens* e, int32_t* values_per_thread);
/* Time `steps` steps of the ensemble in each tile family (16, 8, 4) on its own members and keep
 * the fastest; the members' fields and the Philox step counter are restored afterwards.
 * ms_per_step[3] (may be NULL): ms per step of the families 16, 8, 4; *best (may be NULL): the
 * family kept. Needs gt_ens_set_fields; allocates a copy of the members' fields for the call.
 * Synchronous. */
int gt_ens_autotune(gt_ens* e, int32_t steps, double* ms_per_step, int32_t* best);
const char* gt_ens_last_error(const gt_ens* e);

/* ---- tangent-linear model and discrete adjoint (no counterpart in the reference) ----
 * For the Lawson RK2 step (split or not) followed by the LCG kick, on grids
 * n <= GT_ADJ_MAX_N; gt_adj_gradient and gt_tlm_run also take handles of the
 * Lawson RK4 step (the single-step calls below are RK2 only). The state space is the stored half-spectrum with the real
 * inner product <a, b> = sum Re(conj(a) b); the parameters are the state and
 * the forcing amplitude famp (the phases follow the reference's LCG). */
#define GT_ADJ_MAX_N 4096

/* J(z) = sum over kmin <= |k| <= kmax of fac |z|^2 / |k|^alpha (fac = 1/2 on
 * the kx=0 and Nyquist columns, the weights of src/diagnostics.f90:150-156).
 * J: host; grad: device dJ/dz or NULL. Synchronous. */
int gt_objective(gt_handle* h, const double* z, double kmin, double kmax, double* J, double* grad);
/* One tangent-linear step: z advances exactly as gt_step_rk2 + gt_forcing(z, seed);
 * dz advances by the derivative of that step plus dfamp times the kick pattern
 * of the same LCG draws. *seed advances as in gt_forcing. work: 8 device fields. */
int gt_tlm_step_rk2(gt_handle* h, double* z, double* dz, double dfamp, int32_t* seed, double* const* work);
/* Stage state w = P0 e (z + dt/2 N(z)) of the RK2 step from z (work: 3 fields). */
int gt_adj_stage(gt_handle* h, const double* z, double* w, double* const* work);
/* Adjoint of one RK2 step + kick: z = state at the step start, w = its stage
 * state (gt_adj_stage), lam = dJ/d(state after the kick) on entry and dJ/dz on
 * return; when gfamp != NULL, dJ/dfamp of this kick (LCG state `seed` before it)
 * is added to *gfamp (host; synchronous). work: 6 device fields. */
int gt_adj_step_rk2(gt_handle* h, const double* z, const double* w, double* lam, int32_t seed,
                    double* gfamp, double* const* work);
/* Gradient of J(z after nsteps of RK2 or RK4 + kick from seed, the handle's
 * integrator) with respect to z0 and famp: a forward sweep that stores a
 * checkpoint every K steps, then a backward sweep that recomputes each
 * segment's stage states from its checkpoint and runs the step adjoint back
 * over it. Outputs: J and *grad_famp (host), grad_z0 and zT (device; zT may be
 * NULL), times_ms[2] = forward / backward sweep times (may be NULL). Allocates
 * with cudaMalloc for the duration of the call: RK2 ceil(nsteps/K) + 2K + 8
 * fields and, when the memory is there, the physical u+iv and q of the 2K
 * recomputed stages of a segment (24 N^2 bytes each), which spare the adjoint
 * passes three of their transforms; RK4 ceil(nsteps/K) + 4K + 12 fields and,
 * likewise, the physical fields of its 4K recomputed stage evaluations.
 * Synchronous. */
int gt_adj_gradient(gt_handle* h, const double* z0, int32_t nsteps, int32_t seed, int32_t K,
                    double kmin, double kmax, double* J, double* grad_z0, double* grad_famp,
                    double* zT, double* times_ms);
/* Memory of gt_adj_gradient's kept segments. The forward sweep always keeps its
 * last segment whole (the stage states and the physical u+iv and q of every
 * stage evaluation: RK2 2 fields + 48 N^2 bytes per step, RK4 4 fields +
 * 96 N^2 bytes), which is the storage the backward sweep needs to recompute a
 * segment anyway. With `bytes` > 0 it keeps as many of its last segments whole
 * as fit in `bytes` (at least one), and the backward sweep recomputes only the
 * earlier ones from their checkpoints: memory against recomputation. Default 0
 * (one segment). No counterpart in the reference. */
int gt_adj_set_memory(gt_handle* h, int64_t bytes);
int gt_adj_get_memory(const gt_handle* h, int64_t* bytes);
/* Tangent-linear run: J and its derivative dJ along (dz0, dfamp) after nsteps
 * of the handle's integrator (RK2 or RK4) + kick. */
int gt_tlm_run(gt_handle* h, const double* z0, const double* dz0, double dfamp, int32_t nsteps,
               int32_t seed, double kmin, double kmax, double* J, double* dJ);

/* ---- diagnostics (src/diagnostics.f90:5-179) --------------------------- */

/* Shell spectra, fluxes and global budgets of z (and of znl = nlt(z) for the
 * fluxes). z, znl: device fields. Outputs are HOST arrays of NBIN doubles:
 *   sp, sz   energy / enstrophy spectra, already divided by dk (spectrum)
 *   fle, flz energy / enstrophy flux Pi(k) = suffix sums (fluxes)
 *   glob[6]  = { ee, zz, disz_nu, disz_mu, dise_nu, dise_mu } (glob)
 * Any output pointer may be NULL to skip it. Synchronous (returns once the
 * host arrays are filled). Reductions are deterministic (fixed order). */
int gt_diag(gt_handle* h, const double* z, const double* znl,
            double* sp, double* sz, double* fle, double* flz, double* glob);

/* Largest grid size gt_diag_static accepts (its scratch is sized for it). */
#define GT_DIAG_STATIC_MAX_N 2048

/* gt_diag for callers that cannot allocate device memory. No counterpart in
 * the reference. It serves a driver whose device arrays all live in OpenACC
 * data regions or in another runtime's memory pool sized to fill the GPU, and
 * host code that must not call cudaMalloc/cudaFree between steps (they
 * synchronise the whole device). It needs no gt_handle, allocates nothing and
 * keeps its scratch (~2.3 MB) in a static device array that every GPU loading
 * the library holds until the process exits.
 *   p        the run parameters (n <= GT_DIAG_STATIC_MAX_N, else GT_ERR_ARG)
 *   z, znl   device fields as for gt_diag
 *   sp..glob DEVICE output arrays (NBIN doubles; glob 6), any may be NULL
 *   stream   CUDA stream of the work (NULL = legacy default stream)
 * Asynchronous: returns after enqueueing. No NaN/Inf check. Every call made
 * outside a stream capture looks up the scratch address on the current device
 * (so a cudaDeviceReset between calls is harmless); a call on a capturing
 * stream reuses the address of the device's last earlier call and fails with
 * GT_ERR_STATE if there was none, so make the first call on a device before
 * any stream capture. All calls share the scratch: calls that overlap on the
 * GPU race. Errors are reported through gt_last_error(NULL). */
int gt_diag_static(const gt_params* p, const double* z, const double* znl,
                   double* sp, double* sz, double* fle, double* flz, double* glob,
                   void* cuda_stream);

/* ---- launch timing (benchmarks) ---------------------------------------- */

/* Kernel classes timed by gt_profile: the three passes of the nonlinear term, the forcing
 * kick, the diagnostics, and everything else (transforms, trunc, produ). */
#define GT_PROF_NLT_COLINV 0
#define GT_PROF_NLT_ROW 1
#define GT_PROF_NLT_COLFWD 2
#define GT_PROF_FORCING 3
#define GT_PROF_DIAG 4
#define GT_PROF_OTHER 5
#define GT_PROF_NLT_COLFWD_INV 6 /* pass C of a stage fused with pass A of the next */
#define GT_PROF_KINDS 7

/* No counterpart in the reference (its only timer is a wall clock around the whole run,
 * src/main.f90:191-193). enable=1: record a CUDA event pair on the handle's stream around
 * every later kernel launch; enable=0: stop. */
int gt_profile(gt_handle* h, int enable);
/* Synchronises the stream, returns per class the summed kernel time (ms) and the number of
 * launches since the last read, and resets both. ms, launches: GT_PROF_KINDS entries. */
int gt_profile_read(gt_handle* h, double* ms, int64_t* launches);

/* ---- launch variants and the autotuner ---------------------------------- */

/* No counterpart in the reference, whose transforms are cuFFT plans (src/fft_dir.f90,
 * src/fft_inv.f90) that the library tunes internally. The three passes of the nonlinear
 * term come in GT_NVARIANTS launch shapes: 0 = 16 values per thread, several columns/rows per
 * block (large grids); 1 = 8 values per thread, one column/row per block (n <= 8192);
 * 2 = 4 values per thread, one column/row per block (n <= 1024, for small latency-bound
 * grids); 3 and 4 = 4 and 8 values per thread with the independent transforms of a column
 * (u, v, q; A, B) run side by side by three thread groups of the block (n <= 1024); 5 = 2
 * values per thread, one column per block (32 <= n <= 512). The variants differ only in the
 * radix decomposition of the transforms, so their results agree to rounding (relative
 * differences of order 1e-15 per step). */
#define GT_NVARIANTS 6
/* The row pass takes its own launch variant, numbered like the column variants: 0, 1, 2 =
 * 16, 8, 4 values per thread; 3, 4, 5 = 4, 8 and 2 values per thread with the u + i v and q
 * transforms of a row run side by side by two thread groups (3, 4: n <= 1024; 5: 32 <= n <= 512). */
#define GT_NROW_VARIANTS 6
/* 1 if launch variant `variant` exists for grid size n, else 0 (host only, no GPU needed). */
int gt_variant_supported(int32_t n, int32_t variant);
int gt_row_variant_supported(int32_t n, int32_t row_variant);
/* Select the variant used by every later call of h, for the column and the row passes alike
 * (GT_ERR_ARG if unsupported). */
int gt_set_variant(gt_handle* h, int32_t variant);
int gt_get_variant(const gt_handle* h, int32_t* variant);
/* Select the column and row variants separately. */
int gt_set_variants(gt_handle* h, int32_t col_variant, int32_t row_variant);
int gt_get_variants(const gt_handle* h, int32_t* col_variant, int32_t* row_variant);
/* Field-split column passes (N <= 2048, column variants with one column per CTA and no
 * thread groups: 0 from N = 1024, 1, 2, 5): each CTA transforms one field of one column, so a
 * column pass has 3 (pass A) or 2 (pass C) work units per column and the SMs finish together;
 * q then lives in the handle's scratch field. on = 1: pass C's epilogue is run by the column's
 * CTA that finishes second, which reads the other field back through L2 (a per-column counter);
 * on = 2: the column's two pass C CTAs form one 2-CTA cluster, exchange halves through
 * distributed shared memory and each run the epilogue for half of the rows. On (2) by default;
 * gt_set_col_split(h, 0) returns to one CTA per column. gt_get_col_split reports the mode that
 * runs with the handle's current size and column variant (0 where the split passes do not
 * apply). Results are the same to rounding. */
int gt_set_col_split(gt_handle* h, int32_t on);
int gt_get_col_split(const gt_handle* h, int32_t* active);
/* Programmatic dependent launch of the pass kernels (nonlinear term, tangent-linear, adjoint):
 * each such launch may begin while the previous kernel on the handle's stream drains, and the
 * kernel waits for that kernel's completion before it touches memory, so results do not change.
 * It hides the launch gap between consecutive passes. On by default; off while the handle times
 * its launches (gt_profile). The final pass C of a step with the fused kick, which waits for the
 * side stream's increments, always launches the ordinary way. */
int gt_set_pdl(gt_handle* h, int32_t on);
int gt_get_pdl(const gt_handle* h, int32_t* on);
/* CUDA graphs of the steps (gt_step_rk2, gt_step_rk4 and their _forced forms). No counterpart in
 * the reference. A step is a dozen short launches; with graphs on (the default), each step is
 * captured once per set of fields and launch settings into a CUDA graph of the handle and
 * replayed as one launch (up to 8 graphs per handle, the least recently used evicted), which
 * takes the per-launch host work off the step. Results are bit-identical to the direct launches. The forced
 * steps' LCG state is written into the kick kernel's node before each replay. Steps run as
 * direct launches while the handle times its launches (gt_profile), while the handle's stream
 * is itself being captured, after a capture failed, and once a handle that cycles through more
 * field sets than it keeps graphs for has captured 16 times with fewer than two replays per
 * capture (gt_get_graphs then reports 0; gt_set_graphs(h, 1) tries again).
 * gt_set_graphs(h, 0) frees the handle's graphs. */
int gt_set_graphs(gt_handle* h, int32_t on);
int gt_get_graphs(const gt_handle* h, int32_t* on);
/* Time `steps` steps of the handle's integrator (RK2 or RK4) on zero fields of its own
 * (allocated and freed here, 5 fields; nothing when only one variant exists): first every
 * supported column variant with its own row tiles, then the other row variants under each of
 * the two fastest column variants, then (where the field-split column passes ran) the best pair
 * with one CTA per column, turning the split off if that is faster. Keeps the fastest pair;
 * returns, per column variant, its best ms per step over the row variants tried with it in
 * ms_per_step[GT_NVARIANTS] (-1 for unsupported variants) and the column choice in *best
 * (either pointer may be null; gt_get_variants gives the pair). Synchronous. */
int gt_autotune(gt_handle* h, int32_t steps, double* ms_per_step, int32_t* best);

#ifdef __cplusplus
}
#endif

#endif /* GTURBO_H */
