/*
 * CPU oracle for the MPDATA advection step — TEST INFRASTRUCTURE ONLY.
 *
 * A strict-IEEE (no FMA contraction, no fast-math, left-to-right evaluation)
 * C++ restatement of the reference's MPDATA hot path, written stage by stage
 * from the reference's Fortran sources:
 *   upwind            advection/src_algorithms/upwind3d-gpubc.f90:101-198
 *   standard antidiff advection/src_algorithms/antidiff3d-standard-gpubc.f90:59-462
 *   gauge antidiff    advection/src_algorithms/antidiff3d-gauge-gpubc.f90:71-430
 *   point operators   advection/src_algorithms/mpdataoperators.inc:50-96
 *   halo/BC helpers   advection/src_algorithms/mpdataoperators.inc:253-287,479-584,673-947,1034-1086
 *   predictor         advection/src_algorithms/module_velprd.f90:15-89,166-520
 *   state shift       advection/src_algorithms/velprd_driver.f90:254-270
 *   Courant control   advection/src_algorithms/velprd_driver.f90:16-252,
 *                     common/diagutils.f90:588-672
 *   dispatcher        advection/src_drivers/advec.f90:116-244
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * and only as the checker / the timed CPU baseline.  The product path never
 * links or calls it.
 *
 * Parity pinning: the reference ships one known answer (the 59^3 rotating
 * sphere "Error L2 norm" 0.0028, advection_dwarf_test_modular.f90:157-158);
 * the oracle reproduces it (tests/test_oracle_cpu.py).  No Fortran toolchain
 * exists here or on the GPU host, so field-level parity against the
 * reference binary itself is unpinned beyond the KAT.
 *
 * Arrays are Fortran column-major with the reference's halo extents:
 *   psi-shaped  (1-ih:np+ih,   1-ih:mp+ih,   1-ih:lp+ih)
 *   u1          (1-ih:np+1+ih, 1-ih:mp+ih,   1-ih:lp+ih)
 *   u2          (1-ih:np+ih,   1-ih:mp+1+ih, 1-ih:lp+ih)
 *   u3          (1-ih:np+ih,   1-ih:mp+ih,   1-ih:lp+1+ih)
 *   bcx(mp,lp,2), bcy(np,lp,2)
 *
 * Boundary flags per axis: ibc = 0 is the reference's single-rank rule (open
 * x/y with Dirichlet bcx/bcy halos and zero antidiffusive wall flux; z walls
 * with the mirrored-flux rule f(1)=-f(2), f(lp+1)=-f(lp)); ibc = 1 is a clean
 * periodic wrap with period n on that axis.
 */
#ifndef MPDATA_ORACLE_H
#define MPDATA_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int np, mp, lp, ih;
  int ibcx, ibcy, ibcz;
} orc_grid;

/* advec_dwarf (advec.f90:116-244): legacyoptmode 4 = upwind + antidiffusion,
 * 6 = upwind only; t_adv 1 = gauge, 2 = standard.  iord >= 2 is the number of
 * MPDATA passes (the reference hard-wires 2; >= 3 follows the published MPDATA
 * recursion), nonos = 1 enables the FCT limiter (always on in the reference). */
int orc_advec_dwarf_f64(const orc_grid* g, int legacyoptmode, int t_adv, int iord, int nonos,
                        double* x, const double* x_lr, const double* x_bt,
                        const double* uadv, const double* vadv, const double* wadv,
                        const double* rhr, const double* rhoadv);
int orc_advec_dwarf_f32(const orc_grid* g, int legacyoptmode, int t_adv, int iord, int nonos,
                        float* x, const float* x_lr, const float* x_bt,
                        const float* uadv, const float* vadv, const float* wadv,
                        const float* rhr, const float* rhoadv);

/* Repeated steps (nsteps calls of the above), for timing and long parity runs. */
int orc_advec_steps_f64(const orc_grid* g, int nsteps, int legacyoptmode, int t_adv, int iord,
                        int nonos, double* x, const double* x_lr, const double* x_bt,
                        const double* uadv, const double* vadv, const double* wadv,
                        const double* rhr, const double* rhoadv);
int orc_advec_steps_f32(const orc_grid* g, int nsteps, int legacyoptmode, int t_adv, int iord,
                        int nonos, float* x, const float* x_lr, const float* x_bt,
                        const float* uadv, const float* vadv, const float* wadv,
                        const float* rhr, const float* rhoadv);

/* upwind3d_gpubc alone (upwind3d-gpubc.f90:101-198): writes xant interior. */
int orc_upwind_f64(const orc_grid* g, const double* x, const double* bcx, const double* bcy,
                   const double* u1, const double* u2, const double* u3, const double* rhr,
                   const double* h, double* xant);

/* Velocity predictor velprd_traj0 + velprdA_to_C (module_velprd.f90:15-89,166-364)
 * followed by the driver's level shift (velprd_driver.f90:254-270).
 * ox/oy/oz hold three psi-shaped levels back to back (0: n, 1: n+1/2 out,
 * 2: n-1 momenta); u/v/w (physical velocities, three levels) may be NULL. */
int orc_velprd_f64(const orc_grid* g, double* ox, double* oy, double* oz, double* u, double* v,
                   double* w, const double* h, double dxi, double dyi, double dzi, double dt,
                   double dt_ratio, double* u1, double* u2, double* u3);
int orc_velprd_f32(const orc_grid* g, float* ox, float* oy, float* oz, float* u, float* v,
                   float* w, const float* h, float dxi, float dyi, float dzi, float dt,
                   float dt_ratio, float* u1, float* u2, float* u3);

/* compute_courants (common/diagutils.f90:588-672): cr[0..6] = cr3d, crxy, crxz,
 * cryz, crx, cry, crz.  ntimelevel 1: |dt*dxi*ox(level 0)|; 2: |ox(level 1)/h|. */
int orc_compute_courants_f64(const orc_grid* g, int ntimelevel, double* ox, double* oy, double* oz,
                             const double* h, double dxi, double dyi, double dzi, double dt, double* cr);
int orc_compute_courants_f32(const orc_grid* g, int ntimelevel, float* ox, float* oy, float* oz,
                             const float* h, float dxi, float dyi, float dzi, float dt, float* cr);
/* velprd_driver (advection/src_algorithms/velprd_driver.f90:16-270): Courant
 * control (substepping, adaptive dt, n or n+1/2 diagnosis, split rule), the
 * predictor and the level roll.  diag (9 doubles, may be NULL): the last seven
 * Courant maxima, cr_for_dt, dt_ratio.  Returns 0, -2 (both substepping and
 * adaptivity), -9 (Courant above 10 per substep, or not finite). */
int orc_velprd_driver_f64(const orc_grid* g, int* nsubsteps, int* nsubsteps_o, int lsubstepping,
                          double* dtn, double* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf,
                          double crmaxlim, double dtmax, double* ox, double* oy, double* oz, double* u,
                          double* v, double* w, double* uadv, double* vadv, double* wadv, const double* h,
                          double dxi, double dyi, double dzi, double dt, double* diag);
int orc_velprd_driver_f32(const orc_grid* g, int* nsubsteps, int* nsubsteps_o, int lsubstepping,
                          float* dtn, float* dtnold, int ltimeadapt, int lvertsplit, int lcrdiag_nphlf,
                          float crmaxlim, float dtmax, float* ox, float* oy, float* oz, float* u, float* v,
                          float* w, float* uadv, float* vadv, float* wadv, const float* h, float dxi,
                          float dyi, float dzi, float dt, double* diag);

/* velprdA_to_C_ver2 (module_velprd.f90:366-520): A-grid Courant numbers (psi
 * shaped, halos overwritten by the one-sided extrapolation) -> C grid. */
int orc_a_to_c_f64(const orc_grid* g, double* uadv, double* vadv, double* wadv, double* u1,
                   double* u2, double* u3);

/* mpdata3d_rho_gauge_gpubc (mpdata3d-rho-gauge-gpubc.f90:23-622): predictor,
 * upwind keeping its fluxes, gauge antidiffusion (iord=2, nonoscillatory),
 * then x_incomp = x*h, pexr1 = x_incomp*pexe, pexr2 = x_incomp,
 * rhr = rhoadv/x_incomp (rhoadv = the input x_incomp), and the mass fluxes
 * u1..u3 = upwind flux + limited antidiffusive flux.  liner=1: upwind only. */
int orc_rho_gauge_f64(const orc_grid* g, double* ox, double* oy, double* oz, double* u, double* v,
                      double* w, double* u1, double* u2, double* u3, double* x_in, double* x_incomp,
                      const double* h, double* rhoadv, double* rhr, const double* pexe, double* pexr1,
                      double* pexr2, const double* bcx, const double* bcy, double dxi, double dyi,
                      double dzi, double dt, double dt_ratio, int liner);

/* Un-checkpointed FP64 adjoint of nsteps MPDATA steps (reverse-mode AD of
 * this oracle's own step; branches of max/min/pp/pn/abs/sign taken at the
 * forward values).  J = 0.5*sum((x_N - target)^2) over the interior; returns
 * J, x_N (may be NULL) and dJ/dx_0 (psi-shaped), dJ/du1..u3 (C-grid shaped)
 * for a velocity held fixed over the steps. */
int orc_adjoint_f64(const orc_grid* g, int t_adv, int iord, int nonos, int nsteps, const double* x0,
                    const double* bcx, const double* bcy, const double* u1, const double* u2,
                    const double* u3, const double* rhr, const double* h, const double* target,
                    double* J, double* xN, double* gx0, double* gu1, double* gu2, double* gu3);

/* The density step of orc_rho_gauge_f64 after its predictor: u1..u3 hold the
 * C-grid Courant numbers on entry and the mass fluxes on exit. */
int orc_rho_step_f64(const orc_grid* g, double* u1, double* u2, double* u3, double* x_in, double* x_incomp,
                     const double* h, double* rhoadv, double* rhr, const double* pexe, double* pexr1,
                     double* pexr2, const double* bcx, const double* bcy, int liner);

/* Reverse-mode AD of the density step after its predictor (the step of
 * orc_rho_gauge_f64 from the C-grid Courant numbers on): the outputs psi,
 * x_incomp, pexr1, pexr2, rhr (interiors) and the mass fluxes u1..u3 (faces
 * 1..n+1) take the cotangents l_* (NULL: zero); returns dJ/dpsi_in and
 * dJ/dx_incomp_in, dJ/dpexe (interiors, psi-shaped) and dJ/du1..u3 (every
 * element, C-grid shaped).  h, bcx, bcy are constants. */
int orc_rho_adjoint_f64(const orc_grid* g, const double* u1, const double* u2, const double* u3,
                        const double* x_in, const double* x_incomp, const double* h, const double* pexe,
                        const double* bcx, const double* bcy, const double* l_x, const double* l_u1,
                        const double* l_u2, const double* l_u3, const double* l_xinc, const double* l_p1,
                        const double* l_p2, const double* l_rhr, double* g_x, double* g_u1, double* g_u2,
                        double* g_u3, double* g_xinc, double* g_pexe);

/* orc_adjoint_f64 plus the tangent-linear model on the same tape: dJ_tl =
 * sum((x_N - target) * dx_N) for the directions dx0, du1..du3. */
int orc_tangent_adjoint_f64(const orc_grid* g, int t_adv, int iord, int nonos, int nsteps, const double* x0,
                            const double* bcx, const double* bcy, const double* u1, const double* u2,
                            const double* u3, const double* rhr, const double* h, const double* target,
                            double* J, double* xN, double* gx0, double* gu1, double* gu2, double* gu3,
                            const double* dx0, const double* du1, const double* du2, const double* du3,
                            double* dJ_tl);

/* Order of the cross terms' 4-face velocity sums in the pseudo-velocities.
 * 0 (default): the pair order (a(c)+a(c+e)) + (a(c')+a(c'+e)) that the CUDA
 * kernels reproduce bit for bit.  1: left to right in the order the reference
 * writes the terms (antidiff3d-gauge-gpubc.f90:163-203,
 * antidiff3d-standard-gpubc.f90:99-157), to measure the gap between the two. */
void orc_set_literal_sums(int on);

/* Threads used by the OpenMP loops (1 = the serial reference build). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
