/*
 * mpdata.h — C ABI of the GB300-native MPDATA advection step.
 *
 * Drop-in for the hot path of piotrows/advectionHPCtester: the dwarf driver
 * advec_dwarf and the kernels it dispatches to (upwind, standard and gauge
 * antidiffusion with the nonoscillatory limiter, boundary/halo fill), plus the
 * velocity predictor.  Plain pointers and sizes only; every array pointer is a
 * DEVICE (or managed) pointer to a Fortran column-major array with the
 * reference's halo extents:
 *
 *   psi, h, rhr           (1-ih:np+ih,   1-ih:mp+ih,   1-ih:lp+ih)
 *   u1 (C-grid x faces)   (1-ih:np+1+ih, 1-ih:mp+ih,   1-ih:lp+ih)
 *   u2 (C-grid y faces)   (1-ih:np+ih,   1-ih:mp+1+ih, 1-ih:lp+ih)
 *   u3 (C-grid z faces)   (1-ih:np+ih,   1-ih:mp+ih,   1-ih:lp+1+ih)
 *   bcx (mp,lp,2), bcy (np,lp,2)  Dirichlet x/y halo values of psi
 *
 * Boundary flags per axis (ibcx, ibcy, ibcz):
 *   0  the reference's single-rank rule: open x/y walls take psi's halo from
 *      bcx/bcy in the upwind pass and carry zero antidiffusive flux; z walls
 *      use the mirrored-flux rule f(1) = -f(2), f(lp+1) = -f(lp).
 *   1  periodic with period n on that axis (face n+1 is face 1; caller halos
 *      are neither read nor written on that axis).
 *
 * Conventions: every call returns 0 on success or a negative MPDATA_E* code;
 * nothing exits or aborts.  Calls are ordered on the given CUDA stream (NULL
 * = the legacy default stream) and do not synchronise the host, except where
 * stated.  One host thread per workspace at a time.
 */
#ifndef MPDATA_H
#define MPDATA_H

#ifdef __cplusplus
extern "C" {
#endif

#define MPDATA_OK 0
#define MPDATA_E_DIMS -1        /* bad np/mp/lp/ih or boundary flags */
#define MPDATA_E_OPTS -2        /* bad legacyoptmode/t_adv/iord/nonos/precision */
#define MPDATA_E_NULL -3        /* a required pointer is NULL */
#define MPDATA_E_WS -4          /* workspace missing or built for another grid/options */
#define MPDATA_E_CUDA -5        /* a CUDA runtime call failed */
#define MPDATA_E_DEVICE -6      /* the device error word is set (non-finite result) */
#define MPDATA_E_UNSUPPORTED -7 /* a reference option outside this library's scope */
#define MPDATA_E_TOO_LARGE -8   /* a fixed size limit: the scratch of mpdata_step_noalloc_f64, a batch
                                   tile list of 2^31 tiles, or a netCDF classic slab of 4 GiB */
#define MPDATA_E_COURANT -9     /* Courant control failed (above the fatal limit, or not finite) */
#define MPDATA_E_IO -10         /* field file missing, unreadable, not netCDF classic, or without the variable */

typedef struct {
  int np, mp, lp, ih;   /* interior cells per axis and halo width (ih >= 1) */
  int ibcx, ibcy, ibcz; /* 0 = reference open/wall rule, 1 = periodic */
} mpdata_grid;

typedef struct {
  int iord;      /* number of MPDATA passes: 1 = upwind only, 2 = the reference, >= 3 extra corrective passes */
  int nonos;     /* 1 = nonoscillatory (FCT) limiter, as the reference always does; 0 = off */
  int gauge;     /* 1 = infinite-gauge form (t_adv=1), 0 = standard form (t_adv=2) */
  int precision; /* 64 = FP64 arithmetic, 32 = FP32 arithmetic */
  int predictor; /* reserved for the fused predictor path; 0 */
} mpdata_opts;

/* Workspace: owns the device scratch that the reference keeps in module
 * globals (scratch_datafields_modular.f90:119-134: xant, v1..3, f1..3,
 * f1ns..f3ns, cp, cn).  Replaces allocate_scratch_mpdata_datafields. */
int mpdata_ws_create(const mpdata_grid* grid, const mpdata_opts* opts, void** ws);
int mpdata_ws_destroy(void* ws);

/* One MPDATA step on psi (in place): upwind3d_gpubc followed by iord-1
 * antidiffusive passes.  Replaces the pair of calls
 *   upwind3d_gpubc   advection/src_algorithms/upwind3d-gpubc.f90:20-201
 *   antidiff3d_gauge_gpubc / antidiff3d_standard_gpubc
 *                    advection/src_algorithms/antidiff3d-gauge-gpubc.f90:14-435
 *                    advection/src_algorithms/antidiff3d-standard-gpubc.f90:14-464
 * as dispatched by advec_dwarf (advection/src_drivers/advec.f90:234-240).
 * h is the reference's rhoadv/h, rhr its rhr.  bcx/bcy may be NULL when the
 * axis is periodic. */
int mpdata_step_f64(void* ws, double* psi, const double* u1, const double* u2, const double* u3,
                    const double* h, const double* rhr, const double* bcx, const double* bcy,
                    void* stream);
int mpdata_step_f32(void* ws, float* psi, const float* u1, const float* u2, const float* u3,
                    const float* h, const float* rhr, const float* bcx, const float* bcy,
                    void* stream);

/* The reference driver itself, same argument order and meaning as
 * advec_dwarf (advection/src_drivers/advec.f90:116-122):
 *   legacyoptmode 4 = upwind + antidiffusion, 6 = upwind only (5 is the
 *   HALOBC upwind, whose body is commented out in the reference: rejected);
 *   t_adv 1 = gauge, 2 = standard; lupdatemulti and lvertsplit are accepted
 *   and, as in the reference GPUBC path, change nothing; ipoles must be 0.
 * x_lr/x_bt are the Dirichlet halo values (bcx/bcy), uadv/vadv/wadv the
 * C-grid Courant numbers, rhr and rhoadv the densities.  A workspace for the
 * grid is created on first use and cached (like the reference's module
 * scratch); mpdata_release_cached frees it.  iord/nonos extend the
 * reference's fixed choice (iord=2, nonoscillatory on): pass 2 and 1 for the
 * reference behaviour. */
int mpdata_advec_dwarf_f64(int legacyoptmode, int t_adv, int lupdatemulti, int lvertsplit,
                           int np, int mp, int lp, int ih, int ipoles, int ibcx, int ibcy,
                           int ibcz, double* x, const double* x_lr, const double* x_bt,
                           const double* uadv, const double* vadv, const double* wadv,
                           const double* rhr, const double* rhoadv, int iord, int nonos,
                           void* stream);
int mpdata_advec_dwarf_f32(int legacyoptmode, int t_adv, int lupdatemulti, int lvertsplit,
                           int np, int mp, int lp, int ih, int ipoles, int ibcx, int ibcy,
                           int ibcz, float* x, const float* x_lr, const float* x_bt,
                           const float* uadv, const float* vadv, const float* wadv,
                           const float* rhr, const float* rhoadv, int iord, int nonos,
                           void* stream);
int mpdata_release_cached(void);

/* Velocity predictor: velprd_traj0 + velprdA_to_C
 * (advection/src_algorithms/module_velprd.f90:15-89,166-364) followed by the
 * level roll of velprd_driver (advection/src_algorithms/velprd_driver.f90:254-270).
 * ox/oy/oz: three psi-shaped levels back to back (0 = n, 1 = n+1/2 written,
 * 2 = momenta at n-1, overwritten with ox0*h for the next step).
 * u/v/w: optional physical velocities with the same three levels (NULL to skip).
 * Writes the C-grid Courant numbers u1/u2/u3 (faces 1..n+1). */
int mpdata_velprd_f64(void* ws, double* ox, double* oy, double* oz, double* u, double* v,
                      double* w, const double* h, double dxi, double dyi, double dzi, double dt,
                      double dt_ratio, double* u1, double* u2, double* u3, void* stream);
int mpdata_velprd_f32(void* ws, float* ox, float* oy, float* oz, float* u, float* v, float* w,
                      const float* h, float dxi, float dyi, float dzi, float dt, float dt_ratio,
                      float* u1, float* u2, float* u3, void* stream);

/* Adjoint of mpdata_velprd_* (no reference code): gradients with respect to
 * the A-grid momenta.  The predictor is linear in the momenta of levels 0
 * and 2 for fixed h, dt and dt_ratio (module_velprd.f90:58-83,197-361, the
 * level roll of velprd_driver.f90:254-270); this is its transpose.  g_u1..g_u3
 * hold dJ/du1..u3 (C-grid shaped, faces 1..n+1).  g_ox/g_oy/g_oz are
 * gradient stacks laid out as ox/oy/oz; on entry level 1 holds dJ/d(level 1)
 * and level 2 dJ/d(the level 2 the roll writes) (zero when J does not read
 * them); on exit level 0 has dJ/d(level 0) ADDED and level 2 holds dJ/d(the
 * level 2 the predictor read), so calls chain backwards over steps like the
 * forward's level roll.  Interior cells only; gradients with respect to h and
 * the physical velocity stacks are not formed. */
int mpdata_velprd_adjoint_f64(void* ws, const double* h, double dxi, double dyi, double dzi, double dt,
                              double dt_ratio, const double* g_u1, const double* g_u2, const double* g_u3,
                              double* g_ox, double* g_oy, double* g_oz, void* stream);
int mpdata_velprd_adjoint_f32(void* ws, const float* h, float dxi, float dyi, float dzi, float dt,
                              float dt_ratio, const float* g_u1, const float* g_u2, const float* g_u3,
                              float* g_ox, float* g_oy, float* g_oz, void* stream);

/* Density step of the dycore, mpdata3d_rho_gauge_gpubc
 * (advection/src_algorithms/mpdata3d-rho-gauge-gpubc.f90:23-622): the
 * predictor (as mpdata_velprd_*), then rhoadv = x_incomp, an upwind pass
 * without rhr that keeps its fluxes, gauge antidiffusion with the
 * nonoscillatory limiter (workspace iord/nonos; the workspace must be gauge),
 * and the outputs x_incomp = x*h, pexr1 = x_incomp*pexe, pexr2 = x_incomp,
 * rhr = rhoadv/x_incomp and the mass fluxes u1..u3 = upwind flux + limited
 * antidiffusive flux (faces 1..n+1, overwriting the Courant numbers).
 * liner=1 stops after the upwind pass (:594-606). */
int mpdata_rho_gauge_f64(void* ws, double* ox, double* oy, double* oz, double* u, double* v,
                         double* w, double* u1, double* u2, double* u3, double* x_in,
                         double* x_incomp, const double* h, double* rhoadv, double* rhr,
                         const double* pexe, double* pexr1, double* pexr2, const double* bcx,
                         const double* bcy, double dxi, double dyi, double dzi, double dt,
                         double dt_ratio, int liner, void* stream);
int mpdata_rho_gauge_f32(void* ws, float* ox, float* oy, float* oz, float* u, float* v, float* w,
                         float* u1, float* u2, float* u3, float* x_in, float* x_incomp,
                         const float* h, float* rhoadv, float* rhr, const float* pexe, float* pexr1,
                         float* pexr2, const float* bcx, const float* bcy, float dxi, float dyi,
                         float dzi, float dt, float dt_ratio, int liner, void* stream);

/* ---- adjoint ---------------------------------------------------------------
 * No reference code: the hand-written reverse of the step (infinite-gauge
 * and standard forms, every corrective pass of iord 2 to 8, limiter on or
 * off), every branch differentiated at the forward values.  iord=1:
 * MPDATA_E_UNSUPPORTED.  The workspace's adjoint arena holds 21*(iord-1)+13
 * extra fields (the forward records and accumulators of every pass).
 *
 * mpdata_step_adjoint_*: psi_in is the field at the start of the step (not
 * modified); on entry lambda holds dJ/dpsi after the step (psi-shaped,
 * interior used), on exit dJ/dpsi before it; dJ/du1..u3 of this step are
 * ADDED into g_u1..g_u3 (C-grid shaped).  The forward step is recomputed
 * pass by pass into the workspace's adjoint arena.  Accumulation uses atomic adds, so results
 * match the FP64 reference adjoint to rounding, not bit for bit.
 *
 * mpdata_adjoint_run_*: J = 0.5*sum((psi_N - target)^2) after nsteps steps
 * with velocities held fixed; psi holds psi_0 on entry and psi_N on exit;
 * g_psi0 receives dJ/dpsi_0 and g_u1..g_u3 accumulate dJ/du.  States are
 * checkpointed every `interval` steps (0 = ceil(sqrt(nsteps))) and each
 * segment is recomputed in the reverse sweep.  When interval-1 extra record
 * arenas (15*(iord-1) fields each) fit in half of the free device memory,
 * the recomputation records every step of the segment once and the reverse
 * kernels read those records; otherwise each step adjoint records its own
 * step again.  peak_bytes (may be NULL) receives the device memory the run
 * holds.  Synchronises the stream. */
int mpdata_step_adjoint_f64(void* ws, const double* psi_in, const double* u1, const double* u2,
                            const double* u3, const double* h, const double* rhr, const double* bcx,
                            const double* bcy, double* lambda, double* g_u1, double* g_u2,
                            double* g_u3, void* stream);
int mpdata_step_adjoint_f32(void* ws, const float* psi_in, const float* u1, const float* u2,
                            const float* u3, const float* h, const float* rhr, const float* bcx,
                            const float* bcy, float* lambda, float* g_u1, float* g_u2, float* g_u3,
                            void* stream);
/* Adjoint of the density step after its predictor: the reverse of
 * mpdata_rho_gauge_* from the C-grid Courant numbers u1..u3 it advects with
 * (the predictor's output; mpdata_velprd_adjoint_* carries dJ/du on to the
 * momenta).  Inputs as the forward read them: u1..u3, x_in (psi at the start
 * of the step), x_incomp (its input, which the step copies into rhoadv), h,
 * pexe, bcx, bcy.  Cotangents of the step's outputs: lambda (dJ/dpsi after
 * the step; on exit dJ/dpsi before it), l_u1..l_u3 (the mass fluxes on faces
 * 1..n+1; all three or none), l_xincomp, l_pexr1, l_pexr2, l_rhr (any may be
 * NULL: zero).  g_u1..g_u3 accumulate dJ/du; g_xincomp and g_pexe receive
 * dJ/d(x_incomp input) and dJ/dpexe on the interior.  h is held fixed.  The
 * workspace must be gauge (MPDATA_E_OPTS) with iord >= 2; the forward is
 * recomputed into the adjoint arena.  Results match the FP64 AD oracle to
 * rounding. */
int mpdata_rho_gauge_adjoint_f64(void* ws, const double* u1, const double* u2, const double* u3,
                                 const double* x_in, const double* x_incomp, const double* h,
                                 const double* pexe, const double* bcx, const double* bcy, double* lambda,
                                 const double* l_u1, const double* l_u2, const double* l_u3,
                                 const double* l_xincomp, const double* l_pexr1, const double* l_pexr2,
                                 const double* l_rhr, double* g_u1, double* g_u2, double* g_u3,
                                 double* g_xincomp, double* g_pexe, void* stream);
int mpdata_rho_gauge_adjoint_f32(void* ws, const float* u1, const float* u2, const float* u3,
                                 const float* x_in, const float* x_incomp, const float* h,
                                 const float* pexe, const float* bcx, const float* bcy, float* lambda,
                                 const float* l_u1, const float* l_u2, const float* l_u3,
                                 const float* l_xincomp, const float* l_pexr1, const float* l_pexr2,
                                 const float* l_rhr, float* g_u1, float* g_u2, float* g_u3,
                                 float* g_xincomp, float* g_pexe, void* stream);
int mpdata_adjoint_run_f64(void* ws, int nsteps, int interval, double* psi, const double* u1,
                           const double* u2, const double* u3, const double* h, const double* rhr,
                           const double* bcx, const double* bcy, const double* target, double* J,
                           double* g_psi0, double* g_u1, double* g_u2, double* g_u3,
                           long long* peak_bytes, void* stream);
int mpdata_adjoint_run_f32(void* ws, int nsteps, int interval, float* psi, const float* u1,
                           const float* u2, const float* u3, const float* h, const float* rhr,
                           const float* bcx, const float* bcy, const float* target, double* J,
                           float* g_psi0, float* g_u1, float* g_u2, float* g_u3,
                           long long* peak_bytes, void* stream);

/* Device error word of a workspace (bit 0: a non-finite value was produced
 * by the last checked step).  Synchronises the workspace's last stream. */
int mpdata_ws_error(void* ws, int* error_word);
/* Limiter-bound check of the metric "limiter bounds never violated": the
 * number of interior cells of psi (caller layout, the workspace's precision)
 * outside [mn - tol, mx + tol], where mn/mx are the running extrema the
 * nonoscillatory limiter kept during the workspace's last step (x_in and every
 * pass's stars).  The workspace must have nonos = 1 and iord >= 3 (iord 2
 * keeps no extrema: MPDATA_E_UNSUPPORTED).  With h = rhr = 1 the step's
 * output lies inside the bounds; otherwise the bounds apply to x before the
 * rhr scaling.  Synchronises the stream. */
int mpdata_ws_bound_violations(void* ws, const void* psi, double tol, long long* count, void* stream);

/* Number of kernels this library launched since process start (all
 * workspaces), for launch accounting. */
long long mpdata_launch_count(void);

/* Per-stage kernel timing (replaces the reference's TIMERSCUDA counters,
 * common/mpi_parallel.f90:7256-7338, without a host sync per timer).
 * enable=1: record a CUDA event pair on the launching stream around every
 * kernel of this workspace; enable=0: stop and discard.
 * mpdata_ws_stage_times synchronises on the recorded events and returns the
 * accumulated milliseconds and launch counts per stage (nstages entries,
 * see mpdata_stage_name); the return value is the number of stages. */
int mpdata_ws_profile(void* ws, int enable);
int mpdata_ws_stage_times(void* ws, int nstages, double* total_ms, long long* launches);
const char* mpdata_stage_name(int stage);

/* ---- batches -------------------------------------------------------------
 * Many problems advanced together with ONE launch per stage (a step is a
 * fixed sequence of about ten persistent launches, replayable as one CUDA
 * graph).  Covers
 *  - the reference's multi-tracer step CE_advection, which advects up to 12
 *    fields that share one velocity with one fused upwind kernel and one
 *    antidiffusion per field, the form chosen per field group
 *    (advection/src_drivers/advection_CEtimestep_twostep_GPUBC.f90:27-376,
 *    3186-3494): problems with the same velocity_group share u1..u3, h, rhr
 *    and the scratch derived from them (computed once per group);
 *  - independent domains of uneven sizes (one velocity_group each).
 * All problems share ih, iord, nonos and precision; each has its own grid,
 * boundary flags and form.  Array pointers follow mpdata_step_*. */
typedef struct {
  int np, mp, lp;
  int ibcx, ibcy, ibcz;
  int gauge;          /* 1 = infinite gauge (t_adv=1), 0 = standard (t_adv=2) */
  int velocity_group; /* problems with equal ids share the velocity and densities */
} mpdata_problem;

int mpdata_batch_create(int nprob, const mpdata_problem* probs, int ih, int iord, int nonos,
                        int precision, void** batch);
int mpdata_batch_destroy(void* batch);
/* Arrays of problem `prob` (device pointers, float or double as the batch).
 * Pointers are uploaded with the next step; they may change between steps. */
int mpdata_batch_set(void* batch, int prob, void* psi, const void* u1, const void* u2,
                     const void* u3, const void* h, const void* rhr, const void* bcx,
                     const void* bcy);
/* One step of every problem (in place on each psi), ordered on `stream`. */
int mpdata_batch_step(void* batch, void* stream);
/* enable=1: capture the step's launches into a CUDA graph on the next step
 * and replay the graph afterwards (one graph launch per step). */
int mpdata_batch_graph(void* batch, int enable);
/* Autotuner: times every candidate tile shape (block of bx*by cells) on
 * this batch with steps that write scratch only (psi untouched), keeps the
 * fastest, and caches it for batches of the same signature (precision, iord,
 * nonos, total cells, problem count).  Synchronises the stream. */
int mpdata_batch_tune(void* batch, void* stream, int* bx, int* by);
/* Sets the tile shape (block of bx*by cells, a multiple of 32 and at most
 * 256 threads) without timing, e.g. a shape tuned earlier.  No reference
 * counterpart.  Drops a captured graph.  MPDATA_E_OPTS for an invalid shape.
 * Synchronises the stream. */
int mpdata_batch_set_shape(void* batch, int bx, int by, void* stream);
int mpdata_batch_profile(void* batch, int enable);
int mpdata_batch_stage_times(void* batch, int nstages, double* total_ms, long long* launches);

/* ---- FP64 compensated reductions ------------------------------------------
 * Global sums over the interior in FP64 Neumaier summation, replacing the
 * reference's globsum and norms (common/mpi_parallel.f90:826-880,
 * advection/src_testdata/advection_test_setup.f90:472-617).  Both
 * synchronise `stream` and return host values.
 * mass = sum(h*psi), or sum(h*psi/rhr) when rhr is not NULL. */
int mpdata_mass_f64(const mpdata_grid* grid, const double* psi, const double* h, const double* rhr,
                    double* mass, void* stream);
int mpdata_mass_f32(const mpdata_grid* grid, const float* psi, const float* h, const float* rhr,
                    double* mass, void* stream);
/* Error of field a against reference b (each FP32 or FP64, psi-shaped):
 * out[0] = max|a-b|, out[1] = ||a-b||_2, out[2] = max|b|, out[3] = ||b||_2. */
int mpdata_error_norms(const mpdata_grid* grid, const void* a, int a_is_f64, const void* b,
                       int b_is_f64, double* out, void* stream);

/* ---- Courant control of the predictor ------------------------------------
 * compute_courants (common/diagutils.f90:588-672): cr[0..6] = the maxima over
 * the interior of cr3d, crxy, crxz, cryz, crx, cry, crz.  ntimelevel 1 uses
 * |dt*dxi*ox(level 0)| (and y, z alike), 2 uses |ox(level 1)/h|.  ox/oy/oz are
 * the three-level momentum stacks (1-ih:np+ih, 1-ih:mp+ih, 1-ih:lp+ih, 0:2),
 * h psi-shaped.  Synchronises the stream (the reference's globmax does too).
 * ntimelevel other than 1 or 2: MPDATA_E_OPTS (the reference STOPs). */
int mpdata_compute_courants_f64(double* cr, const double* ox, const double* oy, const double* oz,
                                const double* h, int ntimelevel, double dxi, double dyi, double dzi,
                                double dt, int np, int mp, int lp, int ih, void* stream);
int mpdata_compute_courants_f32(float* cr, const float* ox, const float* oy, const float* oz,
                                const float* h, int ntimelevel, float dxi, float dyi, float dzi,
                                float dt, int np, int mp, int lp, int ih, void* stream);
/* velprd_driver (advection/src_algorithms/velprd_driver.f90:16-270), same
 * argument order: the predictor with substepping (lsubstepping) or an
 * adaptive time step (ltimeadapt), Courant diagnosed at n (lcrdiag_nphlf=0)
 * or n+1/2, the split-scheme Courant rule and wadv halving (lvertsplit), then
 * the level roll.  nsubsteps, nsubsteps_o, dtn and dtnold are INOUT host
 * scalars; u/v/w (physical velocity stacks) may be NULL.  diag, when not NULL,
 * receives the last cr3d, crxy, crxz, cryz, crx, cry, crz, cr_for_dt and
 * dt_ratio.  Synchronises the stream once per Courant evaluation.  Both
 * lsubstepping and ltimeadapt: MPDATA_E_OPTS; Courant above 10 per substep
 * while substepping, or a non-finite Courant number: MPDATA_E_COURANT. */
int mpdata_velprd_driver_f64(int* nsubsteps, int* nsubsteps_o, int lsubstepping, double* dtn,
                             double* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf,
                             double crmaxlim, double dtmax, double* ox, double* oy, double* oz,
                             double* u, double* v, double* w, double* uadv, double* vadv,
                             double* wadv, const double* h, int ipoles, int ibcx, int ibcy, int ibcz,
                             int np, int mp, int lp, int ih, double dxi, double dyi, double dzi,
                             double dt, double* diag, void* stream);
int mpdata_velprd_driver_f32(int* nsubsteps, int* nsubsteps_o, int lsubstepping, float* dtn,
                             float* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf,
                             float crmaxlim, float dtmax, float* ox, float* oy, float* oz, float* u,
                             float* v, float* w, float* uadv, float* vadv, float* wadv,
                             const float* h, int ipoles, int ibcx, int ibcy, int ibcz, int np, int mp,
                             int lp, int ih, float dxi, float dyi, float dzi, float dt, double* diag,
                             void* stream);

/* ---- field output and input (netCDF classic, 64-bit offset) --------------
 * pnet_out_chunk (common/mpi_parallel.f90:7481-8176), single rank, same
 * argument order plus on_device (1: var is a device pointer, 0: host) and
 * stream.  var has extents n+ia*imem+2*ih per axis (psi-shaped for imem 0).
 * imode: 0/1 the interior as float/double (x,y,z,t); 2-4 the staggered
 * block var(1:n+ia) as double with dimensions n+ia; 6-8 the right, top, sky
 * halo strips at offset ih of 2*ih-long dimensions and 9 var(n-ih+1:n) at
 * offset ih on each axis (what one rank writes); 10/13 the xy plane k = ia3 /
 * k = 1 as double (x,y,t); 11/12 the xz plane j = ia2 / yz plane i = ia1
 * through single precision into double (x,z,t) / (y,z,t); 20/21/22 the z, y,
 * x lines through (ia1,ia2), (ia1,ia3), (ia2,ia3) as float; 30 a float (t)
 * variable, never written; 34 the interior as float (x,y,z); 35 the plane
 * k = 1-ih as double (x,y).  A plane or line whose fixed index has
 * (ia-1)/n != 0 lies on another rank: nothing is written.  Other modes return
 * MPDATA_E_UNSUPPORTED.  At ifrmd == 0 the file, the dimensions the mode uses
 * (x, y, z with the mode's lengths, t unlimited) and the variable are created
 * if absent; existing dimensions are reused, and a write that does not fit
 * the variable or the array returns MPDATA_E_DIMS.  Values convert to the
 * variable's type.  Frames between the last record and ifrmd hold the netCDF
 * default fill value, as do the parts of a slab no call wrote.  A variable's
 * slab must stay below 4 GiB (MPDATA_E_TOO_LARGE).  Files are readable by
 * any netCDF-3 reader.  Synchronises the stream. */
int mpdata_pnet_out_chunk_f64(const char* var_name, const char* file_name, int imode, int ia1,
                              int ia2, int ia3, int ifrmd, int imem, const double* var, int np,
                              int mp, int lp, int ih, int on_device, void* stream);
int mpdata_pnet_out_chunk_f32(const char* var_name, const char* file_name, int imode, int ia1,
                              int ia2, int ia3, int ifrmd, int imem, const float* var, int np,
                              int mp, int lp, int ih, int on_device, void* stream);
/* No counterpart in the reference (its restarts read netCDF through
 * PnetCDF): frame ifrmd of a float or double (x,y,z[,t]) variable into the
 * interior of a psi-shaped var (halo untouched), converted to the array's
 * precision.  Synchronises the stream. */
int mpdata_pnet_in_chunk_f64(const char* var_name, const char* file_name, int ifrmd, double* var,
                             int np, int mp, int lp, int ih, int on_device, void* stream);
int mpdata_pnet_in_chunk_f32(const char* var_name, const char* file_name, int ifrmd, float* var,
                             int np, int mp, int lp, int ih, int on_device, void* stream);

/* ---- a step that allocates nothing ----------------------------------------
 * No counterpart in the reference.  For callers that must not have the
 * library allocate device memory (a model that reserves its device memory
 * up front through its own pool, or whose memory use is fixed at start-up):
 * the FP64 step of mpdata_step_f64 without a workspace.  Its scratch is one
 * file-scope device array sized for MPDATA_NOALLOC_MAX_CELLS interior cells
 * (about 5 MB, held on every GPU that loads the library until exit); larger
 * grids return MPDATA_E_TOO_LARGE.  No cudaMalloc/cudaFree is called.  The
 * first call on a device looks up the array's device address, so make it
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU race, so order them (one stream, or synchronise).  Nothing needs
 * clearing between calls.  opts->precision must be 64.  The address is kept
 * for the life of the process: do not call it on a device after
 * cudaDeviceReset there (the array may then live at another address). */
#define MPDATA_NOALLOC_MAX_CELLS 32768
int mpdata_step_noalloc_f64(const mpdata_grid* grid, const mpdata_opts* opts, double* psi,
                            const double* u1, const double* u2, const double* u3, const double* h,
                            const double* rhr, const double* bcx, const double* bcy, void* stream);

const char* mpdata_strerror(int code);
const char* mpdata_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MPDATA_H */
