/*
 * imodel_swm.h -- C ABI of the GB300 TRSK shallow-water time step.
 *
 * This is the seam a Fortran host reaches through iso_c_binding in place of
 * the module procedures of iModel's shallow-water model:
 *
 *   reference call                                  replaced by
 *   ---------------------------------------------   ---------------------------
 *   initialize_gridprop   src/swm.f90:979-1041      imodel_swm_create
 *   ode_rk4 (time loop)   src/swm.f90:249, :2600     imodel_swm_step / _advance
 *   tendency              src/swm.f90:2416-2598      imodel_swm_tendency
 *   sumf_areas, calc_energies, error_calc
 *                         src/swm.f90:3394, :2686, :3492
 *                                                    imodel_swm_diagnostics / _errors
 *   vecrecon_trsk_tg      src/interpack.f90:3852    imodel_swm_trsk_tangent
 *   print* + stop on errors (swm_operators.f90:82-85, :1604-1606,
 *                          swm.f90:331-341)          int32 status codes below
 *
 * All functions return 0 on success and a positive IMODEL_SWM_E* code on
 * failure; none of them aborts or exits.  imodel_swm_last_error() returns a
 * one-line description of the last failure on a handle.
 *
 * Mesh arrays follow the reference's grid_structure (src/datastruct.f90:
 * 121-560): indices are 1-based, per-cell lists are padded to 6 entries in
 * counter-clockwise order (edge j lies between triangles j-1 and j), and
 * "[n][k]" arrays are the Fortran (k, n) column-major layout, i.e. C row-major
 * [n][k].  Lengths and areas are on the unit sphere as the reference stores
 * them.  The library copies everything it needs during create; the caller may
 * free the mesh arrays afterwards.
 *
 * Threading: a handle must not be used from two threads at once.  Separate
 * handles may be used concurrently.
 */
#ifndef IMODEL_SWM_H
#define IMODEL_SWM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define IMODEL_SWM_OK 0
#define IMODEL_SWM_EINVAL 1     /* bad argument or inconsistent mesh          */
#define IMODEL_SWM_ECUDA 2      /* CUDA runtime error (message has details)   */
#define IMODEL_SWM_EBLOWUP 3    /* NaN/Inf in the state (swm.f90:331-341)     */
#define IMODEL_SWM_EDIVZERO 4   /* |h_tr| < eps/1e5 in the PV division
                                   (swm_operators.f90:1604-1606)              */
#define IMODEL_SWM_ENOMEM 5     /* device allocation failed                   */
#define IMODEL_SWM_ESTATE 6     /* call order violated (no state set, ...)    */
#define IMODEL_SWM_ENODEV 7     /* no CUDA device available                   */
#define IMODEL_SWM_ETOOBIG 8    /* input longer than a fixed-size buffer holds */

/* ---- precision modes --------------------------------------------------- */
#define IMODEL_SWM_FP64 0 /* reference operation order, FP64 everywhere      */
#define IMODEL_SWM_FP32 1 /* FP32 state and operators, FP64 integrals        */

/* ---- method wrappers (swm.par's mtdwrapper, swm_data.f90:446-507) ------ */
#define IMODEL_SWM_TRSK10 0 /* trsk interpolation, TRSK Coriolis and K      */
#define IMODEL_SWM_PXT16 1  /* bary interpolation (scalar_hx2tr, tr2ed),
                               pered Coriolis, Perot K (perhx)            */
#define IMODEL_SWM_GASS18 2 /* gass: h_tr from the edges (scalar_edtr2trcc),
                               rhombus PV q_ed, Coriolis with the PV of the
                               connecting edge, TRSK K                    */
#define IMODEL_SWM_DTRED 3  /* mtdwrapper "none" with trsk interpolation and
                               K and coriolis_reconmtd "dtred" (dual
                               triangle Perot reconstruction)             */

/* ---- mesh (copied from grid_structure) --------------------------------- */
typedef struct imodel_swm_mesh {
  int32_t nv, ne, nt;
  /* cells (Voronoi / hexagon-pentagon), datastruct.f90:121-160, :287-400 */
  const int32_t *nnb;          /* [nv]      v%nnb                         */
  const int32_t *v_nb;         /* [nv][6]   v%nb   (neighbour cells)       */
  const int32_t *v_ed;         /* [nv][6]   v%ed   (edges, ccw)            */
  const int32_t *v_tr;         /* [nv][6]   v%tr   (triangles, ccw)        */
  const int32_t *hx_ttgout;    /* [nv][6]   hx%ttgout (+-1)                */
  const int32_t *hx_tnrccw;    /* [nv][6]   hx%tnrccw (+-1)                */
  const double *hx_areag;      /* [nv]      hx%areag                       */
  const double *hx_hxtr_area;  /* [nv][6]   hx%hxtr_area (kite / areag)    */
  const double *hx_trskw;      /* [nv][6][6] hx%trskw(i,j) at [c][j][i]    */
  const double *v_p;           /* [nv][3]   v%p                            */
  const double *v_lat;         /* [nv]      v%lat                          */
  /* triangle edges (HTC velocity points), datastruct.f90:161-211 */
  const int32_t *ed_v;         /* [ne][2]   ed%v  (cells; edhx%sh = ed%v)  */
  const int32_t *ed_sh;        /* [ne][2]   ed%sh (triangles)              */
  const double *ed_leng;       /* [ne]      ed%leng                        */
  const double *edhx_leng;     /* [ne]      edhx%leng                      */
  const double *ed_c;          /* [ne][3]   ed%c%p                         */
  const double *ed_c_lat;      /* [ne]      ed%c%lat                       */
  const double *ed_tg;         /* [ne][3]   ed%tg                          */
  const double *ed_nr;         /* [ne][3]   ed%nr                          */
  /* triangles, datastruct.f90:212-286 */
  const int32_t *tr_v;         /* [nt][3]   tr%v                           */
  const int32_t *tr_ed;        /* [nt][3]   tr%ed                          */
  const int32_t *tr_tg;        /* [nt][3]   tr%tg (+-1)                    */
  const double *tr_areag;      /* [nt]      tr%areag                       */
  const double *tr_trhx_area;  /* [nt][3]   tr%trhx_area                   */
  const double *tr_c_lat;      /* [nt]      tr%c%lat                       */
  /* physical constants (constants.f90:55-67) */
  double erad, grav, omega;
} imodel_swm_mesh;

/* ---- options (par/swm.par subset for the HTC/geo path) ----------------- */
typedef struct imodel_swm_opts {
  int32_t precision;  /* IMODEL_SWM_FP64 or IMODEL_SWM_FP32                 */
  int32_t testcase;   /* reference testcase number: q_tr=0 if <2 and momeq=0
                         if <=1 (swm.f90:2469-2471, :2592-2594)            */
  const double *bt;   /* [nv] bottom topography (m) or NULL for flat        */
  double h_ref;       /* FP32 mode: h is stored as h - h_ref in FP32.
                         0 selects the area mean of the first state set.   */
  int32_t device;     /* CUDA device ordinal                                */
  int32_t learned;    /* 0 off; 1 the per-step learned correction of the
                         TRSK reconstruction (FP32 handles; the network runs
                         once per step on the stencil velocities); 2 learned
                         TRSK weights: at create the network corrects each
                         cell's kite fractions from local geometry and the
                         TRSK weights are rebuilt from them, so the scheme
                         keeps TRSK's structure and a step costs a plain
                         step (trsk10; FP32 handles guarded as below, FP64
                         handles unguarded)                                */
  const void *mlp_weights;  /* packed MLP parameters (see imodel_mlp.h)    */
  size_t mlp_bytes;
  double drift_bound; /* relative total-energy drift above which the
                         learned correction is switched off (0 = 1e-3); it
                         is also switched off when max |u| exceeds 3x its
                         value when the state was set or, for the per-step
                         correction (learned = 1), grows by more than 10 %
                         within one check interval.  Checked every 32
                         steps; the interval that failed is stepped again
                         with the plain scheme                           */
  int32_t scheme;     /* IMODEL_SWM_TRSK10 (0) ... IMODEL_SWM_DTRED; the
                         other wrappers need the mesh's ed_nr and ed_c;
                         FP32 handles run every wrapper in every variant
                         (the cell-centred ones with pered's coefficients
                         and gass18's connecting edges by cell, dtred's
                         Perot vectors by triangle); the learned
                         corrections and ensembles take trsk10 only      */
  int32_t fsphere;    /* Coriolis parameter of vort_tr (swm_operators.f90:
                         551-611): 0 f = 2 Omega sin(lat) at the triangle
                         circumcentres; 2 the constant fcte (f-sphere, test
                         cases 33, 35, 40-42).  The linearised branch 1 of
                         the normal-mode cases is not a time step and is
                         refused                                         */
  double fcte;        /* f for fsphere = 2 (s^-1)                          */
  double error_bound; /* FP32 learned corrections: the error proxy's bound
                         (0 = 0.25).  Every 256 steps (and at the first
                         check after a state is set) the momentum tendency
                         of the learned scheme is compared with plain TRSK's
                         on the current state; a relative difference (L2,
                         edge weights l d) above the bound switches the
                         correction off like the energy check: the
                         interval is stepped again with the plain scheme  */
} imodel_swm_opts;

/* ---- diagnostics (swm.f90:293-322, :2686-2752, :3394-3440) ------------- */
typedef struct imodel_swm_diag {
  double mass;          /* sumf_areas(h) = sum A_i h_i / sum A_i           */
  double penergy;       /* sum A_i g h_i (h_i/2 + b_i)                      */
  double kenergy;       /* sum_e 1/2 l_e d_e h_e u_e^2 (h_e of the last
                           tendency evaluation, as calc_energies uses)     */
  double tenergy;       /* penergy + kenergy                               */
  double availenergy;   /* tenergy - unavailable potential energy          */
  double pot_enstrophy; /* sum_t A_t h_t q_t^2 / 2 (not in the reference)  */
  double rms_div;       /* sqrt(sumfsq_areas(div u)) of the last tendency  */
  double max_div;       /* max |div u|                                     */
  int32_t learned_active; /* 1 while the learned correction is applied     */
  int32_t nan_found;      /* 1 if h or u holds NaN/Inf                      */
} imodel_swm_diag;

/* Creates a handle: copies the mesh, reorders cells along a space-filling
 * curve, builds the padded-CSR connectivity and uploads everything.  On
 * failure *handle is still set, so that imodel_swm_last_error() can explain
 * the failure; it must be released with imodel_swm_destroy() either way. */
int imodel_swm_create(const imodel_swm_mesh *m, const imodel_swm_opts *o,
                      void **handle);

/* Runs nsteps classic RK4 steps (swm.f90:2600-2683) of length dt seconds.
 * h_io[nv] and u_io[ne] (host, FP64, reference ordering) are read on entry
 * and overwritten with the state after nsteps steps.  nsteps > 1 replays a
 * CUDA graph of one step.  Arrays in page-locked memory (cudaMallocHost,
 * cudaHostRegister) that wholly cover nv and ne values are read and written
 * in place by the library's kernels over the host link; pageable arrays are
 * copied through a staging buffer (slower).  The same holds for
 * imodel_swm_set_state and imodel_swm_get_state. */
int imodel_swm_step(void *handle, double *h_io, double *u_io, double dt,
                    int32_t nsteps);

/* One evaluation of tendency(h, u, masseq, momeq) (swm.f90:2416) on host
 * arrays.  Leaves the handle's current state untouched. */
int imodel_swm_tendency(void *handle, const double *h, const double *u,
                        double *masseq, double *momeq);

/* Global integrals of the current state, FP64 with compensated summation. */
int imodel_swm_diagnostics(void *handle, imodel_swm_diag *out);

/* error_calc (swm.f90:3492-3543) of the current state against host
 * reference fields.  out = {Linf_rel_h, L2_rel_h, Linf_h,
 *                           Linf_rel_u, L2_rel_u, Linf_u}. */
int imodel_swm_errors(void *handle, const double *h_ref, const double *u_ref,
                      double out[6]);

/* Tangential velocity reconstructed by TRSK at every edge, along ed%nr
 * (vecrecon_trsk_tg, interpack.f90:3852-3976, var%pos == 6). */
int imodel_swm_trsk_tangent(void *handle, const double *u, double *utg);

int imodel_swm_destroy(void *handle);
const char *imodel_swm_last_error(void *handle);

/* ---- device-resident extensions ---------------------------------------- *
 * A host that keeps the state on the GPU between calls (and a benchmark that
 * measures the kernels alone) uploads once, advances, and reads back when it
 * needs the fields.  These have no counterpart in the reference. */
int imodel_swm_set_state(void *handle, const double *h, const double *u);
int imodel_swm_get_state(void *handle, double *h, double *u);
int imodel_swm_advance(void *handle, double dt, int32_t nsteps);
/* FP32 launch tuning (the project's autotuner): times nsteps graph-replayed
 * steps of every fusion variant and block size on the current state, keeps
 * the fastest and restores the state.  choice = {variant, block size of the
 * triangle, edge pre-pass, cell and edge kernels, gather groups of the
 * learned-correction kernel}; variant 0 uses the 10-entry edge stencil,
 * variant 1 the cell-centred TRSK sum, variant 2 the same with triangle
 * records holding 16-bit indices (bit-identical results); the last entry is
 * 2, 3 or 4 with the
 * learned correction on (its kernel has 6 warp groups, the rest run the
 * epilogue) and 0 without it.  The FP64 path has a single configuration and
 * returns it. */
int imodel_swm_autotune(void *handle, double dt, int32_t nsteps, int32_t choice[6]);
/* Applies a choice returned by imodel_swm_autotune (e.g. cached per grid). */
int imodel_swm_set_tuning(void *handle, const int32_t choice[6]);
/* Laplacian diffusion (K2_max) and hyperdiffusion (K4_max) of the momentum
 * with constant coefficients ("const" branch of swm.f90:169-205), in m^2/s
 * and m^4/s; 0 switches a term off.  The momentum tendency gains
 * + grad(K div u) - grad_tg(K_tr zeta) (diffusion_ed,
 * swm_operators.f90:855-895) and, with K4 > 0, minus the same operator
 * applied twice with sqrt(K4) (hyperdiffusion_ed, :930-975; the Laplacian
 * term then also uses sqrt(K4), as the reference's coefficients do).  Needs
 * the mesh's ed_nr.  May be called at any time; applies from the next step. */
int imodel_swm_set_diffusion(void *handle, double k2, double k4);
/* The same terms with per-cell coefficient fields (nv values in the mesh's
 * cell order, m^2/s and m^4/s; NULL switches a term off), as the "align" and
 * "diam" branches of swm.f90:169-205 form them (alignment_coef,
 * diameter_coef, swm_operators.f90:977-1069): K_tr is the kite-weighted
 * scalar_hx2tr of the field, and with k4_hx both coefficients are the square
 * roots.  Values must be finite and >= 0. */
int imodel_swm_set_diffusion_fields(void *handle, const double *k2_hx, const double *k4_hx);
/* PV stabilisation pv_stab = "apvm" (swm.par; swm_data.f90:548) with
 * parameter pvspar (0 switches it off): before the Coriolis term each edge's
 * PV becomes q_ed - pvspar dt (grad q(t1) + grad q(t2)) . (v(c1) + v(c2)),
 * grad q the Perot reconstruction at the triangles of grad_tr2ed(q_tr) and v
 * that of u at the cells (apvm, swm_operators.f90:1465-1543; called at
 * swm.f90:2557-2559).  dt is the run's time step, which the reference's
 * tendency reads from its module: pass the dt the steps use.  FP32 handles
 * keep their variant: variant 0 applies the correction in its edge
 * pre-pass, variants 1 and 2 run that pre-pass before their cell kernel,
 * which then reads the edges' PV; it combines with the learned corrections.
 * Needs the mesh's ed_nr and ed_c.  May be called at any time; applies from
 * the next step. */
int imodel_swm_set_apvm(void *handle, double pvspar, double dt);
/* The kite fractions hxtr_area[nv][6] and TRSK weights trskw[nv][6][6]
 * (trskw(i, j) at [c][j][i], the mesh's layout) a handle created with
 * learned = 2 steps with: the reference's hx%hxtr_area corrected by the
 * network, and calc_trisk_weights (interpack.f90:3978-4098) of them.  A host
 * that puts them into its grid_structure runs the same scheme on the CPU.
 * IMODEL_SWM_ESTATE for other handles.  No counterpart in the reference. */
int imodel_swm_learned_weights(void *handle, double *hxtr_area, double *trskw);
/* The error proxy (see imodel_swm_opts.error_bound) as last measured: the
 * relative L2 difference between the learned scheme's momentum tendency and
 * plain TRSK's; -1 before the first measurement.  IMODEL_SWM_ESTATE for a
 * handle without a guarded learned correction.  No counterpart in the
 * reference. */
int imodel_swm_learned_error_proxy(void *handle, double *value);
/* Test hook with no counterpart in the reference and no GPU use: builds the
 * device layout of mesh m for `scheme` on the host with `nthreads` threads
 * (0 = all) and returns a 64-bit FNV-1a digest of every layout array, so
 * that a test can show the layout does not depend on the thread count. */
int imodel_swm_test_layout_digest(const imodel_swm_mesh *m, int32_t scheme, int32_t nthreads,
                                  uint64_t *digest);
/* Test hook with no counterpart in the reference: when after > 0, the
 * after-th device allocation made by any handle from now on fails with
 * IMODEL_SWM_ENOMEM as if the device were full (0 switches the injection
 * off).  It lets tests check that a failed set-up (set_apvm,
 * set_diffusion*) leaves the handle stepping correctly without the option. */
int imodel_swm_test_fail_alloc(int32_t after);
/* Launches issued by one advance call for nsteps steps (kernels only). */
int imodel_swm_launch_count(void *handle, int32_t nsteps, int64_t *count);
/* Runs nsteps RK4 steps kernel by kernel (no graph) with CUDA events around
 * each kernel on the handle's stream and returns the average duration in ms
 * of the four kernels of a stage: {triangle (PV), edge pre-pass (h_e, F_e,
 * q_e), cell (div F, K, B, mass update), edge (grad B + TRSK PV flux,
 * momentum update)}.  Advances the state like imodel_swm_advance. */
int imodel_swm_profile(void *handle, double dt, int32_t nsteps, double avg_ms[4]);
/* Name of the kernel that dominates a step (for profilers). */
const char *imodel_swm_main_kernel(void *handle);
/* The CUDA stream (cudaStream_t) all work of the handle is issued on. */
void *imodel_swm_stream(void *handle);

/* ---- ensembles ----------------------------------------------------------- *
 * Many instances of the FP32 step on up to 8 grids (e.g. 64 members on one
 * level and 16 on another) advanced together by ONE persistent cooperative
 * launch.  Members of a grid share its geometry; their states are
 * interleaved member-fastest.  Each grid keeps its own dt and step count; the
 * grids' steps are spread evenly over the launch.  Member results equal the
 * single-run FP32 path (variant 1) bit for bit when both store h against the
 * same reference depth (a grid's reference is the area mean of the first
 * state set on it; other members differ from their own single runs at the
 * 1e-7 level).  No counterpart in the reference, which runs one instance per
 * process. */
int imodel_swm_ensemble_create(const imodel_swm_mesh *meshes, int32_t ngrids,
                               const int32_t *members, int32_t testcase, int32_t device,
                               void **ens);
int imodel_swm_ensemble_set_state(void *ens, int32_t grid, int32_t member, const double *h,
                                  const double *u);
int imodel_swm_ensemble_get_state(void *ens, int32_t grid, int32_t member, double *h,
                                  double *u);
/* dt[ngrids] seconds and nsteps[ngrids] RK4 steps per grid, one launch. */
int imodel_swm_ensemble_advance(void *ens, const double *dt, const int32_t *nsteps);
/* Autotuner of the persistent launch: times nsteps steps per grid for each
 * kernel variant (0: registers unconstrained, 1: at most 64 registers per
 * thread for more resident warps), block size and blocks-per-SM count, keeps
 * the fastest, restores the state.
 * choice = {block size, blocks per SM, variant}. */
int imodel_swm_ensemble_tune(void *ens, const double *dt, int32_t nsteps, int32_t choice[3]);
/* Test hook with no counterpart in the reference: in the next
 * imodel_swm_ensemble_advance launch only, block `block` of the persistent
 * launch leaves before its first grid-wide barrier and every barrier wait
 * gives up after spin_limit polls (about 64 ns each).  The other blocks then
 * time out, the launch ends and the advance returns IMODEL_SWM_ECUDA ("grid
 * barrier timed out"); the ensemble stays usable (set the states again). */
int imodel_swm_ensemble_test_stall(void *ens, int32_t block, int64_t spin_limit);
int imodel_swm_ensemble_destroy(void *ens);
const char *imodel_swm_ensemble_last_error(void *ens);
void *imodel_swm_ensemble_stream(void *ens);

/* Area-weighted sums of one field with no device allocation.  No counterpart
 * in the reference: it is the compensated reduction behind
 * imodel_swm_diagnostics (sumf_areas / sumfsq_areas) for callers that cannot
 * call cudaMalloc -- a host whose device memory is all handed out by another
 * runtime's pool, or a plugin that may only touch the buffers its caller
 * gives it.  Instead of a handle's buffer it uses a 256 KiB block-partials
 * array built into the library (every GPU that loads the library keeps it
 * until the process exits).
 *
 * w, f: device arrays of n doubles (weights, field); out: device array of 4
 * doubles receiving {sum w, sum w*f, sum w*f^2, max |f|}, the sums
 * Neumaier-compensated; a NaN in f makes the maximum NaN as well as the sums.
 * stream: a cudaStream_t (NULL = legacy default stream); the call only
 * enqueues work, out is valid once the stream reaches it.  n may be at most
 * 33,554,432 (4096 blocks x 256 threads x 32 elements); a longer input
 * returns IMODEL_SWM_ETOOBIG and launches nothing.  Runs on the current
 * device.  Its first call on a device (and its first call after another
 * context was made current there) looks up the array's device address
 * (cudaGetSymbolAddress) before it launches anything.  All calls share the
 * one array, and each call overwrites the partials it reads: calls whose work
 * overlaps on the GPU (different streams, or different host threads on one
 * device) race and must be serialised by the caller.  IMODEL_SWM_ECUDA
 * reports a failed launch of this call only; an error the caller left
 * pending in the runtime is neither reported nor cleared. */
int imodel_swm_weighted_sums_noalloc(const double *w, const double *f, int64_t n, double *out,
                                     void *stream);

#ifdef __cplusplus
}
#endif
#endif /* IMODEL_SWM_H */
