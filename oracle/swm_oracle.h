/*
 * swm_oracle.h -- CPU restatement of iModel's TRSK shallow-water step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the correctness oracle and the CPU
 * baseline of the GB300 library; the library never links or calls it.
 * Parity status: the reference is Fortran and no Fortran compiler exists
 * where this was written, so bit-level parity with the reference binary is
 * unpinned; the restatement is pinned instead by the reference's own
 * known-answer tests (Williamson TC2 steady state and its analytic operator
 * values, swm.f90:1205-1326 and :382-734; mimetic identities :628-718).
 */
#ifndef IMODEL_SWM_ORACLE_H
#define IMODEL_SWM_ORACLE_H
#include <stdint.h>
#include "../include/imodel_swm.h"
#ifdef __cplusplus
extern "C" {
#endif

void *oracle_create(const imodel_swm_mesh *m, int32_t testcase, const double *bt,
                    int32_t nthreads);
void oracle_destroy(void *o);
/* Laplacian diffusion / hyperdiffusion with constant coefficients (m^2/s,
 * m^4/s; 0 = off), swm.f90:169-205 and swm_operators.f90:855-975 */
int oracle_set_diffusion(void *o, double k2, double k4);
/* the same with per-cell coefficient fields [nv] (NULL: term off), the
 * "align" / "diam" branches of swm.f90:169-205 */
int oracle_set_diffusion_fields(void *o, const double *k2_hx, const double *k4_hx);
/* pv_stab = "apvm" with parameter pvspar (0 = off) and the run's time step
 * dt, swm_operators.f90:1465-1543 */
int oracle_set_apvm(void *o, double pvspar, double dt);
/* Coriolis parameter: fsphere 0 (2 Omega sin lat) or 2 (constant fcte),
 * vort_tr, swm_operators.f90:592-601 */
int oracle_set_fcor(void *o, int32_t fsphere, double fcte);
/* method wrapper: 0 trsk10, 1 pxt16, 2 gass18, 3 trsk10 with the dtred
 * Coriolis reconstruction (swm_data.f90:446-507) */
int oracle_set_scheme(void *o, int32_t scheme);
int oracle_tendency(void *o, const double *h, const double *u, double *masseq,
                    double *momeq);
int oracle_rk4(void *o, const double *h, const double *u, double *h_new, double *u_new,
               double dt);
int oracle_run(void *o, double *h, double *u, double dt, int32_t nsteps);
int oracle_diagnostics(void *o, const double *h, const double *u, imodel_swm_diag *out);
int oracle_error_calc(void *o, const double *f, const double *fref, int32_t pos,
                      double out[3]);
int oracle_trsk_tangent(void *o, const double *u, double *utg);
int oracle_trsk_weights(const imodel_swm_mesh *m, double *trskw);
int oracle_tc2(const imodel_swm_mesh *m, double *h, double *u);
/* copy an intermediate field of the last tendency call:
 * 0 h_ed, 1 uh, 2 eta, 3 h_tr, 4 q_tr, 5 q_ed, 6 divuh, 7 ke, 8 ghbK,
 * 9 grad_ghbK, 10 uhq_perp, 11 divu, 12 zeta, 13 eta_ed, 14 lapu, 15 lap_lapu,
 * 16 q_grad_ed, 17 h_rhb, 18 vhq_tr [nt][3], 19 v_hx [nv][3] */
int oracle_field(void *o, int32_t which, double *out);

/* the moist shallow-water model (moist_swm.f90) with advmtd = "trsk" and
 * RK4: theta[nv] is the potential temperature the sources read (frozen at
 * its initial value, as in the reference's RK4 path), q0 the saturation
 * scale of its test case */
void *oracle_moist_create(const imodel_swm_mesh *m, int32_t testcase, const double *bt,
                          const double *theta, double q0, int32_t nthreads);
void oracle_moist_destroy(void *o);
int oracle_moist_set_q(void *o, const double *qv, const double *qc, const double *qr);
/* advmtd of the tracer advection: 0 = "trsk" (the default), 1 = "upw1" */
int oracle_moist_set_advection(void *o, int32_t upw1);
/* y = {h[nv], u[ne], htheta, hqv, hqc, hqr, htracer [nv]}, advanced in place */
int oracle_moist_run(void *o, double *const y[7], double dt, int32_t nsteps);

#ifdef __cplusplus
}
#endif
#endif
