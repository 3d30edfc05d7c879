// Shared declarations of the TRSK shallow-water kernels (internal header).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace imodel {

// Device copy of the layout (pointers into one device allocation each).
struct DevMesh {
  int nv, ne, nt;
  double erad, grav;
  // cells
  const int8_t *c_nnb;
  const int32_t *c_ed;
  const double *c_sd, *c_areag, *c_cellarea, *c_bt;
  const float *c_div32, *c_kew32, *c_bt32;
  // edges
  const int32_t *e_v, *e_sh;
  const double *e_leng, *e_dleng, *e_kew, *e_area;
  const float *e_grad32;
  const double *e_sgtg;   // [ne] sign of grad_ed_tg (swm_layout.h)
  const float *e_gtg32;   // [ne] sign / (edhx%leng erad)
  const int8_t *e_nst;
  const int32_t *e_stk;
  const double *e_stw;
  const float *e_stc32;
  // triangles
  const int32_t *t_ed, *t_v;
  const double *t_lt, *t_kite, *t_areag, *t_f;
  const float *t_f32;
  const int4 *t_recA, *t_recB;  // [nt] packed triangle records (swm_layout.h)
  const float4 *t_recC;
  // cell-centred TRSK variant (FP32)
  const int32_t *c_nb, *c_tr;
  const float *c_R32, *c_dg32, *c_inva32;
  const float *c_area32, *e_area32;  // A_i and l_e d_e / 2 in FP32 (drift check)
  const uint32_t *c_meta, *e_vs;
  const int4 *c_pk;     // [6][nv] {edge, neighbour, triangle, kite fraction bits}
  const float2 *c_kd;   // [6][nv] {KE weight, ttgout*d}
  const uint2 *e_vs2;   // [ne] both cell words of an edge
  // the triangle records with 16-bit indices against per-warp bases
  // (variant 2; swm_layout.h): {e0|e1, e2|c0, c1|c2, circ 0}, {circ 1,
  // circ 2, kite 0, kite 1}, {kite 2, f} [nt], warp bases {edge, cell (-1:
  // use the 32-bit records)}
  const uint4 *t_c16A;
  const float4 *t_c16B;
  const float2 *t_c16C;
  const int2 *t_wb;
  // points for the APVM reconstructions (FP64, [3][n], NULL without
  // ed%nr): ed%c%p, tr%c%p (circumcentre), v%p
  const double *e_c, *t_c, *c_p;
  // the FP32 step's APVM weights and projection vectors (swm_layout.h)
  const float *t_apw32, *t_cc32, *c_apw32, *c_p32;
  // geometry of the pxt16, gass18 and dtred method wrappers (FP64, NULL
  // for trsk10; swm_layout.h): barycentric weights [3][nt], circumcentre
  // distances [2][ne], edge areas [3][nt], connecting edges [10][ne], ed%nr
  // [3][ne]
  const double *t_bary, *e_dist, *t_edarea, *e_nr;
  const int32_t *e_stq;
  // their FP32 coefficients (swm_layout.h): q_e weights [2][ne] (pxt16,
  // gass18), dtred's PV-flux coefficients [6][ne]
  const float *e_qw32, *e_dtc32;
  // pxt16's pered coefficients by cell [36][nv] and gass18's outer
  // triangle edges [6][nv] (the cell-centred variants; swm_layout.h)
  const float *c_C32;
  const int32_t *c_gout;
  const float *c_qw32;  // [12][nv] the q_e weights by cell slot (pxt16)
  // dtred's Perot weights by triangle [9][nt], opposite corners [nt], and
  // per edge nr [3][ne] and the triangle weights [2][ne] (swm_layout.h)
  const float *t_dpa32, *e_nr32, *e_dw32;
  const uint8_t *t_dopp;
};

// Launch configuration of the FP32 stage kernels, chosen by the autotuner.
//   variant 0: triangle -> edge pre-pass -> cell -> edge (10-entry stencil)
//   variant 1: triangle -> cell (cell-centred TRSK, writes the PV flux
//              contribution of each cell edge) -> edge (sums two cells)
//   variant 2: variant 1 reading the triangle records with 16-bit indices
//              (40 instead of 52 bytes per triangle)
struct Tune {
  int variant = 1;
  int bs_tri = 256, bs_pre = 256, bs_cell = 256, bs_edge = 256;
  int mlp_gather = 2;  // gather groups of the learned-correction kernel (2..4)
};

struct LearnedDev;

// Laplacian diffusion and hyperdiffusion of the momentum (diffusion_ed,
// hyperdiffusion_ed, swm_operators.f90:855-975; coefficients swm.f90:169-205,
// "const" branch).  lap = grad_ed(K div x) - grad_ed_tg(K_tr zeta(x)) for
// x = u, and for x = lap with hyperdiffusion; the momentum tendency gains
// + lap (K2 > 0) and - lap2 (K4 > 0), in that order.
template <class T>
struct Diffusion {
  bool on = false, k2 = false, k4 = false;
  T *kcv = nullptr;         // [nv] at the cells: K2, or sqrt(K4)
  T *kt = nullptr;          // [nt] at triangles: hx2tr(K2), or sqrt(hx2tr(K4))
  T *coefdiv = nullptr;     // [nv] K div x
  T *coefvort = nullptr;    // [nt] K_tr zeta(x)
  T *lap = nullptr, *lap2 = nullptr;  // [ne]
};

// The anticipated potential vorticity method, apvm (swm_operators.f90:
// 1465-1543): q_ed -= pvspar dt (grad q(t1) + grad q(t2)) . (v(c1) + v(c2)).
template <class T>
struct Apvm {
  bool on = false;
  T coef = T(0);          // pvspar * dt
  T *qg = nullptr;        // [3][nt] Perot reconstruction of grad_tr2ed(q_tr)
  T *vhx = nullptr;       // [3][nv] Perot reconstruction of u at the cells
  T *qge = nullptr;       // [ne] grad_tr2ed(q_tr) (FP64 step)
};

// Working fields of one handle, in the handle's precision T.
template <class T>
struct Work {
  const LearnedDev *learned = nullptr;  // FP32 variants 1, 2: learned correction on
  T *yn_h, *yn_u;    // state at t_n (advanced in place at the last stage)
  T *ya_h, *ya_u;    // stage inputs (ping)
  T *yb_h, *yb_u;    // stage inputs (pong)
  T *acc_h, *acc_u;  // k0 + 2 k1 + 2 k2
  T *q_tr;           // [nt] potential vorticity at triangles
  T *h_ed, *uh, *q_ed;  // [ne]
  T *bern;           // [nv] g (h + b) + K
  T *tend_h, *tend_u;   // tendency outputs (tendency-only evaluations)
  T *zflux;          // [6][nv] cell-centred PV flux of each cell edge (variants 1, 2)
  Diffusion<T> dif;
  Apvm<T> apvm;
  Tune tune;
  int *flags;        // bit 0: PV division by ~0
  // method wrapper (IMODEL_SWM_TRSK10 ... IMODEL_SWM_DTRED; FP64 handles)
  int scheme = 0;
  T *eta_t = nullptr, *h_trs = nullptr;  // [nt] gass18: eta and h_tr for the rhombus PV
  T *vhq = nullptr;                      // [3][nt] dtred: Perot reconstruction of uh, times q
                                         // (FP64, and FP32 variants 1 and 2)
  T h_ref;           // FP32: h is stored as h - h_ref
  int pv_on;         // testcase >= 2: q = eta / h_tr, else q = 0
  int mom_on;        // testcase >= 2: momentum tendency kept, else zeroed
};

// One tendency evaluation (stage < 0: write masseq/momeq to tend_*), or RK4
// stage `stage` (0..3) of classic RK4 reading y_in and writing y_out.
// ev (may be NULL): 5 events recorded before, between and after the four
// kernels of the stage, for per-kernel timing outside graph capture.
void launch_stage64(const DevMesh &M, const Work<double> &W, const double *h_in,
                    const double *u_in, double *h_out, double *u_out, int stage,
                    double dt, cudaStream_t s, cudaEvent_t *ev = nullptr);
// The learned corrections' error proxy: per block part[2 b] = sum w (a -
// b)^2 and part[2 b + 1] = sum w (b - c)^2 over the edges, in FP64, w = l d
// / 2 (e_area32); nblk blocks of 256 threads
void launch_departure(const DevMesh &M, const float *a, const float *b, const float *c,
                      double *part, int nblk, cudaStream_t s);
void launch_stage32(const DevMesh &M, const Work<float> &W, const float *h_in,
                    const float *u_in, float *h_out, float *u_out, int stage, float dt,
                    cudaStream_t s, cudaEvent_t *ev = nullptr);
// The learned TRSK correction inside the FP32 step (mlp.cu): once per step,
// after the first stage's PV, corr[e] = q_e h_e sigma_e y_e is formed from the
// network output; the edge kernel adds it to the momentum tendency of every
// stage of that step.
struct LearnedDev {
  float *p = nullptr;        // FP32 parameters
  uint16_t *img = nullptr;   // BF16 weight images
  // network inputs, one 11,264-byte block per 128-edge tile (LearnedLayout)
  const uint8_t *blocks = nullptr;
  float *corr = nullptr;     // [ne]
  int sms = 0;
};
int learned_prepare(const float *params_host, LearnedDev *L, cudaStream_t s);
void learned_launch(const DevMesh &M, const LearnedDev &L, const float *hd, const float *u,
                    const float *q_tr, float h_ref, int gather_groups, int *err, cudaStream_t s);

// kernel launches of one RK stage; with diffusion on, the edge gradients
// (1 launch, 3 with hyperdiffusion) and, for FP32 variant 0, a first pass of
// K div u and K_tr zeta (1 launch)
inline int launches_per_stage(int precision_fp32, int variant, bool dif_on = false,
                              bool dif_k4 = false, bool apvm_on = false, int scheme = 0) {
  int n = (precision_fp32 && variant >= 1) ? 3 : 4;
  if (!precision_fp32 && scheme == 3) n += 1;  // dtred: the triangle reconstruction of uh q
  if (dif_on) n += (dif_k4 ? 3 : 1) + ((precision_fp32 && variant == 0) ? 1 : 0);
  // FP32 variants 1 and 2: the edge pre-pass for APVM's or gass18's edge PV
  if (precision_fp32 && variant >= 1 && (apvm_on || scheme == 2)) n += 1;
  // the reconstructions
  if (apvm_on) n += precision_fp32 ? 1 : 2;
  return n;
}
// The diffusion coefficients from the cell field kf (device order, FP64;
// NULL: the constant k): kc64 = kf at the cells and kt64 = scalar_hx2tr(kf)
// (kite-area weights) at the triangles, each then sqrt with take_sqrt
// (hyperdiffusion); kc32 / kt32, when not NULL, their FP32 roundings
void launch_dif_coefs(const DevMesh &M, const double *kf, double k, bool take_sqrt, double *kc64,
                      float *kc32, double *kt64, float *kt32, cudaStream_t s);


// One RK stage of the moist shallow-water model (swm_moist.cu).  Tracer k of
// {h theta, h qv, h qc, h qr, h tracer} is advanced when bit k of `active`
// is set; swm != 0 adds the shallow-water terms (the caller has written
// tend_h, tend_u and h_ed with a tendency evaluation of the stage input),
// the thermal momentum source and the water sources.
struct MoistArgs {
  int stage = 0;
  double dt = 0.0;
  int swm = 0, active = 0;
  int upw1 = 0;  // tracer advection: 0 "trsk" (centred), 1 "upw1" (upwind)
  const double *u_in = nullptr, *h_in = nullptr, *tend_u = nullptr, *tend_h = nullptr,
               *h_ed = nullptr;
  double *yn_u = nullptr, *acc_u = nullptr, *u_out = nullptr;
  double *yn_h = nullptr, *acc_h = nullptr, *h_out = nullptr;
  const double *q_in[5] = {};
  double *q_yn[5] = {}, *q_acc[5] = {}, *q_out[5] = {};
  double *uphi = nullptr;  // [5][ne]
  // theta (frozen), exp(20 theta), and qv, qc, qr of the last step [nv]
  const double *th = nullptr, *ex20 = nullptr, *qv = nullptr, *qc = nullptr, *qr = nullptr;
  double q0 = 0.0;
  int *flags = nullptr;
};
void launch_moist_stage(const DevMesh &M, const MoistArgs &A, cudaStream_t s);
void launch_moist_q(int nv, const double *h, const double *hqv, const double *hqc,
                    const double *hqr, double *qv, double *qc, double *qr, int *flags,
                    cudaStream_t s);
// The same in FP32 beside the FP32 step (tendencies of any variant): h as
// h - h_ref, the tracers h q as they are, the geometry's folded FP32
// coefficients; the cells form the tracer fluxes themselves
struct MoistArgs32 {
  int stage = 0;
  float dt = 0.0f;
  int swm = 0, active = 0;
  int upw1 = 0;
  float h_ref = 0.0f;
  const float *u_in = nullptr, *h_in = nullptr, *tend_u = nullptr, *tend_h = nullptr;
  float *yn_u = nullptr, *acc_u = nullptr, *u_out = nullptr;
  float *yn_h = nullptr, *acc_h = nullptr, *h_out = nullptr;
  const float *q_in[5] = {};
  float *q_yn[5] = {}, *q_acc[5] = {}, *q_out[5] = {};
  const float *th = nullptr, *ex20 = nullptr, *qv = nullptr, *qc = nullptr, *qr = nullptr;
  float q0 = 0.0f;
  int *flags = nullptr;
};
void launch_moist_stage32(const DevMesh &M, const MoistArgs32 &A, cudaStream_t s);
void launch_moist_q32(int nv, const float *hd, float h_ref, const float *hqv, const float *hqc,
                      const float *hqr, float *qv, float *qc, float *qr, int *flags,
                      cudaStream_t s);

// reference order <-> device order, with precision conversion
void launch_gather_in(int n, const int32_t *n2o, const double *src, double *dst, double shift,
                      cudaStream_t s);
void launch_gather_in32(int n, const int32_t *n2o, const double *src, float *dst, double shift,
                        cudaStream_t s);
// flags may be NULL; otherwise bit 1 is set when a value is NaN/Inf
void launch_scatter_out(int n, const int32_t *n2o, const double *src, double *dst, double shift,
                        int *flags, cudaStream_t s);
void launch_scatter_out32(int n, const int32_t *n2o, const float *src, double *dst,
                          double shift, int *flags, cudaStream_t s);
// the same conversions straight between a page-locked host array (reference
// order, read or written in order over the host link) and the device state:
// load writes yn, ya and (when not NULL) ck; store raises bit 1 of *flags on
// NaN/Inf
template <class T>
void launch_load_host(int n, const int32_t *o2n, const double *src, T *yn, T *ya, T *ck,
                      double shift, cudaStream_t s);
template <class T>
void launch_store_host(int n, const int32_t *o2n, const T *src, double *dst, double shift,
                       int *flags, cudaStream_t s);


// Compensated FP64 integrals.  Scratch: partial sums, 2 doubles per block
// and quantity; result[kDiagQ] on the device.
constexpr int kDiagQ = 12;
constexpr int kRedBlocks = 608;   // 4 blocks per SM on 152 SMs
constexpr int kRedThreads = 256;
// result indices
enum {
  Q_AREA = 0, Q_AH, Q_PE, Q_AHB, Q_AB2, Q_KE, Q_ENS, Q_ADIV2, Q_MAXDIV, Q_NAN,
  Q_UMAX,  // max |u| over the edges
  Q_SPARE1
};
// energy_only: potential and kinetic energy only (the other entries are 0)
template <class T>
void launch_diag(const DevMesh &M, const Work<T> &W, const T *h, const T *u, const T *hs,
                 const T *us, double *scratch, double *result, cudaStream_t s,
                 bool energy_only = false);
// error_calc partials: {sum A dif^2, sum A ref^2, max|dif|, max|ref|} for h
// then for u.
template <class T>
void launch_errors(const DevMesh &M, const T *h, const T *u, double h_ref, const double *href,
                   const double *uref, double *scratch, double *result, cudaStream_t s);
// vecrecon_trsk_tg at every edge (FP64, reference order); u and utg in
// device order
void launch_trsk_tangent(const DevMesh &M, const double *u, double *utg, cudaStream_t s);

}  // namespace imodel
