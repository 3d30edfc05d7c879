/*
 * imodel_moist.h -- C ABI of the moist shallow-water model on the GPU.
 *
 * Replaces the time loop of iModel's moist shallow-water model
 * (moist_swm_tests, src/moist_swm.f90:1394-1600) with advmtd = "trsk" or
 * "upw1", time_integrator = "rk4" and no monotonic filter:
 *
 *   reference call                                       replaced by
 *   ---------------------------------------------------  ----------------------
 *   initialize_global_moist_swm_vars, mesh set-up        imodel_moist_create
 *   ode_rk4_moist_swm (moist_swm.f90:1819-2011)          imodel_moist_advance
 *     tendency_moist_swm (:1151-1276), source (:1278-1353),
 *     tendency_advection / divhx (highorder.f90:3936-3972, :4901-4983,
 *     div_hx_upw1 :5094-5139)
 *   qv, qc, qr = hq / h after each step (:1531-1533)     inside imodel_moist_advance
 *
 * The shallow-water part is the trsk10 / HTC / geodesic-area tendency of
 * imodel_swm.h, in FP64 in the reference's operation order (bit-equal to
 * the CPU oracle) or in FP32.  Mesh arrays as in imodel_swm.h; status codes
 * IMODEL_SWM_*.
 */
#ifndef IMODEL_MOIST_H
#define IMODEL_MOIST_H
#include <stdint.h>
#include "imodel_swm.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct imodel_moist_opts {
  int32_t testcase;    /* moist test case 1..5: 1 advects the passive tracer
                          alone (h, u and the water fields stay fixed); 2
                          also advects it; 3-5 leave it fixed              */
  const double *bt;    /* [nv] bottom topography (m) or NULL              */
  const double *theta; /* [nv] the potential temperature the sources read
                          (the reference's RK4 path keeps its initial value)*/
  double q0;           /* saturation scale of the test case               */
  int32_t device;      /* CUDA device ordinal                             */
  int32_t advection;   /* advmtd of the tracers: 0 = "trsk" (centred,
                          divhx, highorder.f90:4967-4974), 1 = "upw1"
                          (first-order upwind, div_hx_upw1, :5094-5139)   */
  int32_t precision;   /* IMODEL_SWM_FP64 (0: the reference's operation
                          order, bit-equal to the oracle) or
                          IMODEL_SWM_FP32 (FP32 state, tracers and sources
                          beside the FP32 step; h stored as h - h_ref, h_ref
                          the area-weighted mean of the first state set)  */
} imodel_moist_opts;

int imodel_moist_create(const imodel_swm_mesh *m, const imodel_moist_opts *o, void **handle);
/* y[7] = {h[nv], u[ne], h theta[nv], h qv[nv], h qc[nv], h qr[nv],
 * h tracer[nv]} (host, FP64, reference order); qv, qc, qr [nv] the water
 * fields the first step's sources read. */
int imodel_moist_set_state(void *handle, const double *const y[7], const double *qv,
                           const double *qc, const double *qr);
/* nsteps RK4 steps of dt seconds; after each, qv, qc, qr = hq / h. */
int imodel_moist_advance(void *handle, double dt, int32_t nsteps);
int imodel_moist_get_state(void *handle, double *const y[7]);
int imodel_moist_destroy(void *handle);
const char *imodel_moist_last_error(void *handle);

#ifdef __cplusplus
}
#endif
#endif /* IMODEL_MOIST_H */
