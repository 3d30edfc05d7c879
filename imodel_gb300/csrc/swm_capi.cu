// C ABI of the GB300 TRSK shallow-water step (include/imodel_swm.h).
//
// A handle owns the device copy of the mesh layout, the state buffers of
// classic RK4 and one CUDA stream.  One RK4 step is 4 stages x 4 kernels;
// it is captured once into a CUDA graph per time step length and replayed.
#include <cuda.h>  // pointer-attribute types only; the driver call is resolved at run time
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "imodel_mlp.h"
#include "imodel_moist.h"
#include "imodel_swm.h"
#include "swm_common.cuh"
#include "swm_layout.h"

namespace imodel {
namespace {

struct Handle {
  // gass18 on a grid whose connecting edges do not follow the cells'
  // structure (Layout::gass_cells false): the stencil variant only
  bool v0_only = false;
  std::string err;
  int device = 0;
  int precision = IMODEL_SWM_FP64;
  int testcase = 2;
  int nv = 0, ne = 0, nt = 0;
  double area_cells = 0.0, area_edges = 0.0;  // sum A_i, sum l d / 2
  std::vector<double> h_areag;                 // reference order, for h_ref
  bool href_fixed = false;
  double h_ref = 0.0;
  DevMesh M{};
  std::vector<void *> allocs;
  int32_t *d_cell_n2o = nullptr, *d_edge_n2o = nullptr;
  int32_t *d_cell_o2n = nullptr, *d_edge_o2n = nullptr;
  // cuPointerGetAttribute, for the extent of a caller's page-locked array
  CUresult (*range_attr)(void *, CUpointer_attribute, CUdeviceptr) = nullptr;
  double *d_stage_h = nullptr, *d_stage_u = nullptr;  // FP64, reference order
  double *d_ref_h = nullptr, *d_ref_u = nullptr;      // FP64, device order
  double *d_scratch = nullptr, *d_result = nullptr;
  int *d_flags = nullptr;
  int *h_flags = nullptr;      // pinned
  double *h_result = nullptr;  // pinned
  Work<double> W64{};
  Work<float> W32{};
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0.0;
  bool state_set = false;
  // learned TRSK correction: mode 1 the per-step network (FP32, cell-centred
  // variant), mode 2 the learned TRSK weights (kite fractions corrected once
  // at create)
  LearnedDev learned{};
  int learned_mode = 0;
  bool learned_on = false;      // a guarded learned correction (FP32 handles)
  bool learned_active = false;  // still applied (the drift guard may switch it off)
  // mode 2: the weight-dependent device arrays of the learned and of the
  // plain scheme (the guard's fallback), and host copies of the learned
  // kite fractions and weights (reference layout) for export
  struct WeightSet {
    const double *e_stw = nullptr;
    const float *e_stc32 = nullptr, *c_R32 = nullptr;
    const int4 *c_pk = nullptr;
  } w_learned, w_plain;
  imodel::HVec<double> kite_hxtr, kite_trskw;
  double drift_bound = 1e-3;
  // the error proxy: bound, the learned and the plain momentum tendency
  // ([2][ne]), and the steps left until the next check (<= 0: at the next
  // guard check)
  double error_bound = 0.25;
  float *proxy_u = nullptr;
  int64_t proxy_left = 0;
  double last_proxy = -1.0;  // the last value measured (-1: none yet)
  double te_ref = 0.0, umax_ref = 0.0;
  double umax_last = 0.0;  // max |u| at the start of the current guard interval
  bool te_ref_set = false;
  // state at the start of the current guard interval, restored when the
  // interval ends past the drift bound (or with a non-finite energy)
  float *ck_h = nullptr, *ck_u = nullptr;
  bool ck_fresh = false;  // ck holds yn (written by the page-locked load)
  // the mesh gave ed%nr, which the diffusion terms' tangential gradient needs
  bool dif_ok = false;
  double *d_kt64 = nullptr;  // [nt] FP64 K_tr scratch of an FP32 handle
  double *d_kc64 = nullptr;  // [nv] FP64 K scratch of an FP32 handle
  double *d_kf = nullptr;    // [2][nv] coefficient fields: reference order, device order
  // a second stream for the energy check, which runs beside the write-back
  // of the state in imodel_swm_step
  cudaStream_t side = nullptr;
  cudaEvent_t ev_steps = nullptr, ev_side = nullptr;
};

// steps between two checks of the learned correction's energy drift
constexpr int kGuardSteps = 32;
// the check also fails when max |u| exceeds kUmaxCap times its value when the
// state was set or, for the per-step correction (learned = 1), grows by more
// than kUmaxStep within one interval: its coupling of the stencil edges is
// not antisymmetric, and the mode it grows at a few edges hardly moves the
// total energy before it blows up.  Smooth flows change max |u| far more
// slowly (7.4 % per 256 steps at most in case 5, flow over a mountain), but
// a vigorous one can jump by more than 10 % in 32 steps (level 10, dt 28 s,
// 60 m/s winds, degree-256 spectrum, plain TRSK included); the learned TRSK
// weights keep TRSK's antisymmetry and are judged by energy and the cap only.
constexpr double kUmaxStep = 1.1;
constexpr double kUmaxCap = 3.0;
// steps between two evaluations of the error proxy (two tendencies: about
// 0.2 % of the step time at this spacing)
constexpr int kProxySteps = 256;

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      H->err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
      return e_ == cudaErrorMemoryAllocation ? IMODEL_SWM_ENOMEM : IMODEL_SWM_ECUDA; \
    }                                                                             \
  } while (0)

template <class V, class A>
int upload(Handle *H, const std::vector<V, A> &v, const V **dst) {
  if (v.empty()) {
    *dst = nullptr;
    return IMODEL_SWM_OK;
  }
  void *p = nullptr;
  CK(cudaMalloc(&p, v.size() * sizeof(V)));
  H->allocs.push_back(p);
  CK(cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
  *dst = static_cast<const V *>(p);
  return IMODEL_SWM_OK;
}

// host-side allocation-failure injection for tests: when > 0, the
// allocation that brings the count to zero fails as if the device were full
std::atomic<int> g_fail_alloc_after{0};

template <class T>
int dalloc(Handle *H, T **p, size_t n) {
  void *q = nullptr;
  int after = g_fail_alloc_after.load();
  while (after > 0 && !g_fail_alloc_after.compare_exchange_weak(after, after - 1)) {
  }
  if (after == 1) {
    H->err = "cudaMalloc: out of memory (injected by imodel_swm_test_fail_alloc)";
    return IMODEL_SWM_ENOMEM;
  }
  CK(cudaMalloc(&q, (n > 0 ? n : 1) * sizeof(T)));
  H->allocs.push_back(q);
  CK(cudaMemset(q, 0, (n > 0 ? n : 1) * sizeof(T)));
  *p = static_cast<T *>(q);
  return IMODEL_SWM_OK;
}

template <class T>
int alloc_work(Handle *H, Work<T> &W) {
  int rc;
  T **bufs_v[] = {&W.yn_h, &W.ya_h, &W.yb_h, &W.acc_h, &W.bern, &W.tend_h};
  for (T **b : bufs_v)
    if ((rc = dalloc(H, b, H->nv))) return rc;
  T **bufs_e[] = {&W.yn_u, &W.ya_u, &W.yb_u, &W.acc_u, &W.h_ed, &W.uh, &W.q_ed, &W.tend_u};
  for (T **b : bufs_e)
    if ((rc = dalloc(H, b, H->ne))) return rc;
  if ((rc = dalloc(H, &W.q_tr, H->nt))) return rc;
  W.flags = H->d_flags;
  W.pv_on = H->testcase >= 2 ? 1 : 0;
  W.mom_on = H->testcase > 1 ? 1 : 0;
  W.h_ref = T(0);
  return IMODEL_SWM_OK;
}

int set_error(Handle *H, int code, const std::string &msg) {
  H->err = msg;
  return code;
}

// one RK4 step on the device state (4 stages; swm.f90:2600-2683)
void enqueue_step(Handle *H, double dt) {
  cudaStream_t s = H->stream;
  if (H->precision == IMODEL_SWM_FP64) {
    const Work<double> &W = H->W64;
    launch_stage64(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, 0, dt, s);
    launch_stage64(H->M, W, W.ya_h, W.ya_u, W.yb_h, W.yb_u, 1, dt, s);
    launch_stage64(H->M, W, W.yb_h, W.yb_u, W.ya_h, W.ya_u, 2, dt, s);
    launch_stage64(H->M, W, W.ya_h, W.ya_u, W.yn_h, W.yn_u, 3, dt, s);
  } else {
    const Work<float> &W = H->W32;
    const float fdt = static_cast<float>(dt);
    launch_stage32(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, 0, fdt, s);
    launch_stage32(H->M, W, W.ya_h, W.ya_u, W.yb_h, W.yb_u, 1, fdt, s);
    launch_stage32(H->M, W, W.yb_h, W.yb_u, W.ya_h, W.ya_u, 2, fdt, s);
    launch_stage32(H->M, W, W.ya_h, W.ya_u, W.yn_h, W.yn_u, 3, fdt, s);
  }
}

int ensure_graph(Handle *H, double dt) {
  if (H->graph && H->graph_dt == dt) return IMODEL_SWM_OK;
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step(H, dt);
  CK(cudaStreamEndCapture(H->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&H->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    H->graph = nullptr;
    return set_error(H, IMODEL_SWM_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  H->graph_dt = dt;
  return IMODEL_SWM_OK;
}

// A device address of a caller's host array of `bytes` bytes when the array
// lies wholly inside page-locked memory known to CUDA (cudaMallocHost,
// cudaHostAlloc, cudaHostRegister) and mapped for this handle's device;
// nullptr otherwise, and the array then goes through cudaMemcpyAsync.  The
// extent check keeps a kernel from reaching past the caller's allocation.
void *host_view(Handle *H, const void *p, size_t bytes) {
  if (!H->range_attr || !p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer || a.device != H->device) return nullptr;
  CUdeviceptr start = 0;
  size_t size = 0;
  const CUdeviceptr q = reinterpret_cast<CUdeviceptr>(p);
  if (H->range_attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, q) != CUDA_SUCCESS ||
      H->range_attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, q) != CUDA_SUCCESS)
    return nullptr;
  if (q < start || q - start > size || bytes > size - (q - start)) return nullptr;
  // the device address keeps p's offset inside the allocation
  return static_cast<char *>(a.devicePointer);
}

// host FP64 arrays (reference order) -> device state yn, plus h_ed and the
// "last stage input" ya, as after the reference's initial tendency call
// (swm.f90:214)
int learned_guard(Handle *H, bool *tripped = nullptr, int steps = 0);

// new_run: the state starts a new run (set_state), so the learned correction
// is switched back on and its energy reference is taken again
// the learned correction on or off: mode 1 launches the network inside the
// step, mode 2 points the step at the learned or the plain TRSK weights
void learned_switch(Handle *H, bool on) {
  if (H->learned_mode == 1) {
    H->W32.learned = on ? &H->learned : nullptr;
  } else if (H->learned_mode == 2) {
    const Handle::WeightSet &w = on ? H->w_learned : H->w_plain;
    H->M.e_stw = w.e_stw;
    H->M.e_stc32 = w.e_stc32;
    H->M.c_R32 = w.c_R32;
    H->M.c_pk = w.c_pk;
  }
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
}

int load_state(Handle *H, const double *h, const double *u, bool new_run) {
  if (H->precision == IMODEL_SWM_FP32 && !H->href_fixed) {
    double s = 0.0, a = 0.0;
    for (int i = 0; i < H->nv; ++i) {
      a += H->h_areag[i];
      s += H->h_areag[i] * h[i];
    }
    H->h_ref = s / a;
    H->W32.h_ref = static_cast<float>(H->h_ref);
    H->h_ref = static_cast<double>(H->W32.h_ref);
    H->href_fixed = true;
  }
  const double *hz = static_cast<const double *>(host_view(H, h, sizeof(double) * H->nv));
  const double *uz = static_cast<const double *>(host_view(H, u, sizeof(double) * H->ne));
  if (hz && uz) {
    // page-locked arrays: one kernel per array reads them over the host link
    // in order and writes yn and ya in device order (no staging copy)
    // (and, with the learned correction on, the guard's checkpoint)
    if (H->precision == IMODEL_SWM_FP64) {
      Work<double> &W = H->W64;
      launch_load_host<double>(H->nv, H->d_cell_o2n, hz, W.yn_h, W.ya_h, nullptr, 0.0, H->stream);
      launch_load_host<double>(H->ne, H->d_edge_o2n, uz, W.yn_u, W.ya_u, nullptr, 0.0, H->stream);
      H->ck_fresh = false;
    } else {
      Work<float> &W = H->W32;
      const bool ck = H->learned_on;
      launch_load_host(H->nv, H->d_cell_o2n, hz, W.yn_h, W.ya_h, ck ? H->ck_h : nullptr,
                       H->h_ref, H->stream);
      launch_load_host(H->ne, H->d_edge_o2n, uz, W.yn_u, W.ya_u, ck ? H->ck_u : nullptr, 0.0,
                       H->stream);
      H->ck_fresh = ck;
    }
  } else if (H->precision == IMODEL_SWM_FP64) {
    CK(cudaMemcpyAsync(H->d_stage_h, h, sizeof(double) * H->nv, cudaMemcpyHostToDevice, H->stream));
    CK(cudaMemcpyAsync(H->d_stage_u, u, sizeof(double) * H->ne, cudaMemcpyHostToDevice, H->stream));
    Work<double> &W = H->W64;
    launch_gather_in(H->nv, H->d_cell_n2o, H->d_stage_h, W.yn_h, 0.0, H->stream);
    launch_gather_in(H->ne, H->d_edge_n2o, H->d_stage_u, W.yn_u, 0.0, H->stream);
    CK(cudaMemcpyAsync(W.ya_h, W.yn_h, sizeof(double) * H->nv, cudaMemcpyDeviceToDevice, H->stream));
    CK(cudaMemcpyAsync(W.ya_u, W.yn_u, sizeof(double) * H->ne, cudaMemcpyDeviceToDevice, H->stream));
  } else {
    CK(cudaMemcpyAsync(H->d_stage_h, h, sizeof(double) * H->nv, cudaMemcpyHostToDevice, H->stream));
    CK(cudaMemcpyAsync(H->d_stage_u, u, sizeof(double) * H->ne, cudaMemcpyHostToDevice, H->stream));
    Work<float> &W = H->W32;
    launch_gather_in32(H->nv, H->d_cell_n2o, H->d_stage_h, W.yn_h, H->h_ref, H->stream);
    launch_gather_in32(H->ne, H->d_edge_n2o, H->d_stage_u, W.yn_u, 0.0, H->stream);
    CK(cudaMemcpyAsync(W.ya_h, W.yn_h, sizeof(float) * H->nv, cudaMemcpyDeviceToDevice, H->stream));
    CK(cudaMemcpyAsync(W.ya_u, W.yn_u, sizeof(float) * H->ne, cudaMemcpyDeviceToDevice, H->stream));
  }
  if (!(hz && uz)) H->ck_fresh = false;
  CK(cudaGetLastError());
  H->state_set = true;
  if (H->learned_on && (new_run || !H->te_ref_set)) {
    if (!H->learned_active) {
      H->learned_active = true;
      learned_switch(H, true);
    }
    H->te_ref_set = false;
    H->proxy_left = 0;
    return learned_guard(H);
  }
  return IMODEL_SWM_OK;
}

int store_state(Handle *H, double *h, double *u) {
  double *hz = static_cast<double *>(host_view(H, h, sizeof(double) * H->nv));
  double *uz = static_cast<double *>(host_view(H, u, sizeof(double) * H->ne));
  if (hz && uz) {
    // page-locked arrays: written in order over the host link by the
    // kernels that undo the permutation (no staging copy)
    if (H->precision == IMODEL_SWM_FP64) {
      launch_store_host(H->nv, H->d_cell_o2n, H->W64.yn_h, hz, 0.0, H->d_flags, H->stream);
      launch_store_host(H->ne, H->d_edge_o2n, H->W64.yn_u, uz, 0.0, H->d_flags, H->stream);
    } else {
      launch_store_host(H->nv, H->d_cell_o2n, H->W32.yn_h, hz, H->h_ref, H->d_flags, H->stream);
      launch_store_host(H->ne, H->d_edge_o2n, H->W32.yn_u, uz, 0.0, H->d_flags, H->stream);
    }
    CK(cudaGetLastError());
    return IMODEL_SWM_OK;
  }
  if (H->precision == IMODEL_SWM_FP64) {
    launch_scatter_out(H->nv, H->d_cell_n2o, H->W64.yn_h, H->d_stage_h, 0.0, H->d_flags, H->stream);
    launch_scatter_out(H->ne, H->d_edge_n2o, H->W64.yn_u, H->d_stage_u, 0.0, H->d_flags, H->stream);
  } else {
    launch_scatter_out32(H->nv, H->d_cell_n2o, H->W32.yn_h, H->d_stage_h, H->h_ref, H->d_flags,
                         H->stream);
    launch_scatter_out32(H->ne, H->d_edge_n2o, H->W32.yn_u, H->d_stage_u, 0.0, H->d_flags,
                         H->stream);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h, H->d_stage_h, sizeof(double) * H->nv, cudaMemcpyDeviceToHost, H->stream));
  CK(cudaMemcpyAsync(u, H->d_stage_u, sizeof(double) * H->ne, cudaMemcpyDeviceToHost, H->stream));
  return IMODEL_SWM_OK;
}

// reads and clears the device flags (synchronising the stream)
int read_flags(Handle *H, int *f) {
  CK(cudaMemcpyAsync(H->h_flags, H->d_flags, sizeof(int), cudaMemcpyDeviceToHost, H->stream));
  CK(cudaMemsetAsync(H->d_flags, 0, sizeof(int), H->stream));
  CK(cudaStreamSynchronize(H->stream));
  *f = *H->h_flags;
  return IMODEL_SWM_OK;
}

// maps device flags to a status
int flags_status(Handle *H, int f) {
  if (f & 1)
    return set_error(H, IMODEL_SWM_EDIVZERO,
                     "division by zero in PV (|h_tr| < eps/1e5), as scalar_elem_divide stops");
  if (f & 2) return set_error(H, IMODEL_SWM_EBLOWUP, "state holds NaN or Inf");
  // bits 8 and 16: a bounded wait of the learned-correction network kernel
  // ran out (mlp.cu, mlp_pipe.cuh); the kernel returned without finishing
  // its tiles, so the correction of that step is incomplete
  if (f & (8 | 16))
    return set_error(H, IMODEL_SWM_ECUDA,
                     "the learned-correction kernel's pipeline gave up on a bounded wait");
  return IMODEL_SWM_OK;
}

int check_flags(Handle *H) {
  int f = 0;
  const int rc = read_flags(H, &f);
  return rc ? rc : flags_status(H, f);
}

// total energy of the current state (compensated FP64 integral) and max |u|
// enqueues it on stream s, with the read-back into h_result
int enqueue_energy(Handle *H, cudaStream_t s) {
  if (H->precision == IMODEL_SWM_FP64) {
    auto &W = H->W64;
    launch_diag<double>(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, H->d_scratch, H->d_result, s,
                        true);
  } else {
    auto &W = H->W32;
    launch_diag<float>(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, H->d_scratch, H->d_result, s,
                       true);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(H->h_result, H->d_result, sizeof(double) * kDiagQ, cudaMemcpyDeviceToHost,
                     s));
  return IMODEL_SWM_OK;
}

int total_energy(Handle *H, double *te, double *umax) {
  int rc = enqueue_energy(H, H->stream);
  if (rc) return rc;
  CK(cudaStreamSynchronize(H->stream));
  *te = H->h_result[Q_PE] + H->h_result[Q_KE];
  *umax = H->h_result[Q_UMAX];
  return IMODEL_SWM_OK;
}

// Fallback of the learned correction: once the relative drift of the total
// energy since the state was set exceeds the bound (or the energy is not
// finite), the plain TRSK scheme takes over for the rest of the run.
// *tripped tells the caller that the guard switched the correction off.
// the decision on a measured energy and max |u|; true when it switched the
// correction off
bool guard_decide(Handle *H, double te, double umax) {
  if (!H->te_ref_set) {
    H->te_ref = te;
    H->umax_ref = H->umax_last = umax;
    H->te_ref_set = true;
    return false;
  }
  const double drift = std::fabs(te - H->te_ref) / std::fabs(H->te_ref);
  const bool step_ok = H->learned_mode == 2 || umax <= kUmaxStep * H->umax_last;
  if (drift <= H->drift_bound && step_ok && umax <= kUmaxCap * H->umax_ref) {
    H->umax_last = umax;
    return false;
  }
  H->learned_active = false;
  learned_switch(H, false);
  return true;
}

// The error proxy (opts.error_bound): how far the learned scheme moves the
// PV flux of plain TRSK on the current state, ||T_l - T_p|| / ||T_0 - T_p||
// (L2, edge weights l d), with T_l, T_p the momentum tendencies of the
// learned and the plain scheme and T_0 the plain one with the PV off (-grad
// B), so that the denominator is the plain PV flux itself (the whole
// tendency nearly vanishes on a steady flow).  Without a reference
// solution, how far the network moves the term it corrects is the error it
// can add: the learned weights move it by a few per cent, a network gone
// wrong by far more.  The plain tendencies are launched with local copies
// of the device mesh and work fields, so the handle (and its captured
// graph) keep the learned scheme.  Due every kProxySteps steps.
int error_proxy(Handle *H, int steps, bool *trip) {
  *trip = false;
  H->proxy_left -= steps;
  if (H->proxy_left > 0 || !H->learned_active || H->precision != IMODEL_SWM_FP32) return IMODEL_SWM_OK;
  H->proxy_left = kProxySteps;
  auto &W = H->W32;
  imodel::launch_stage32(H->M, W, W.yn_h, W.yn_u, nullptr, nullptr, -1, 1.0f, H->stream, nullptr);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(H->proxy_u, W.tend_u, sizeof(float) * H->ne, cudaMemcpyDeviceToDevice,
                     H->stream));
  DevMesh Mp = H->M;
  imodel::Work<float> Wp = W;
  if (H->learned_mode == 2) {
    Mp.e_stw = H->w_plain.e_stw;
    Mp.e_stc32 = H->w_plain.e_stc32;
    Mp.c_R32 = H->w_plain.c_R32;
    Mp.c_pk = H->w_plain.c_pk;
  } else {
    Wp.learned = nullptr;
  }
  imodel::launch_stage32(Mp, Wp, W.yn_h, W.yn_u, nullptr, nullptr, -1, 1.0f, H->stream, nullptr);
  float *plain_u = H->proxy_u + H->ne;
  CK(cudaMemcpyAsync(plain_u, W.tend_u, sizeof(float) * H->ne, cudaMemcpyDeviceToDevice,
                     H->stream));
  Wp.pv_on = 0;  // q = 0: the tendency without the PV flux
  imodel::launch_stage32(Mp, Wp, W.yn_h, W.yn_u, nullptr, nullptr, -1, 1.0f, H->stream, nullptr);
  imodel::launch_departure(H->M, H->proxy_u, plain_u, W.tend_u, H->d_scratch, kRedBlocks,
                           H->stream);
  CK(cudaGetLastError());
  std::vector<double> part(2 * static_cast<size_t>(kRedBlocks));
  CK(cudaMemcpyAsync(part.data(), H->d_scratch, sizeof(double) * part.size(),
                     cudaMemcpyDeviceToHost, H->stream));
  CK(cudaStreamSynchronize(H->stream));
  double d2 = 0.0, b2 = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) {
    d2 += part[2 * k];
    b2 += part[2 * k + 1];
  }
  const double dep = b2 > 0.0 ? std::sqrt(d2 / b2) : (d2 > 0.0 ? INFINITY : 0.0);
  H->last_proxy = dep;
  if (!(dep <= H->error_bound)) {
    H->learned_active = false;
    learned_switch(H, false);
    *trip = true;
  }
  return IMODEL_SWM_OK;
}

int learned_guard(Handle *H, bool *tripped, int steps) {
  if (tripped) *tripped = false;
  if (!H->learned_active) return IMODEL_SWM_OK;
  double te = 0.0, umax = 0.0;
  int rc = total_energy(H, &te, &umax);
  if (rc) return rc;
  bool t = guard_decide(H, te, umax);
  if (!t && (rc = error_proxy(H, steps, &t))) return rc;
  if (tripped) *tripped = t;
  return IMODEL_SWM_OK;
}

int launch_steps(Handle *H, double dt, int nsteps) {
  int rc = ensure_graph(H, dt);
  if (rc) return rc;
  H->ck_fresh = false;
  for (int k = 0; k < nsteps; ++k) CK(cudaGraphLaunch(H->graph, H->stream));
  return IMODEL_SWM_OK;
}

// copies the state aside at the start of a guard interval (unless the
// page-locked load already wrote the copy)
int save_checkpoint(Handle *H) {
  if (H->ck_fresh) return IMODEL_SWM_OK;
  auto &W = H->W32;
  CK(cudaMemcpyAsync(H->ck_h, W.yn_h, sizeof(float) * H->nv, cudaMemcpyDeviceToDevice, H->stream));
  CK(cudaMemcpyAsync(H->ck_u, W.yn_u, sizeof(float) * H->ne, cudaMemcpyDeviceToDevice, H->stream));
  H->ck_fresh = true;
  return IMODEL_SWM_OK;
}

// back to the state at the start of the interval
int roll_back(Handle *H) {
  auto &W = H->W32;
  const size_t bh = sizeof(float) * H->nv, bu = sizeof(float) * H->ne;
  CK(cudaMemcpyAsync(W.yn_h, H->ck_h, bh, cudaMemcpyDeviceToDevice, H->stream));
  CK(cudaMemcpyAsync(W.yn_u, H->ck_u, bu, cudaMemcpyDeviceToDevice, H->stream));
  CK(cudaMemcpyAsync(W.ya_h, H->ck_h, bh, cudaMemcpyDeviceToDevice, H->stream));
  CK(cudaMemcpyAsync(W.ya_u, H->ck_u, bu, cudaMemcpyDeviceToDevice, H->stream));
  // flags raised by the rolled-back steps do not describe the state
  CK(cudaMemsetAsync(H->d_flags, 0, sizeof(int), H->stream));
  return IMODEL_SWM_OK;
}

// With the learned correction on, the steps run in guard intervals: the
// state is copied aside, the interval is stepped and the energy checked;
// an interval that ends past the drift bound is rolled back and stepped
// again with the plain scheme, so no corrected step that broke the bound
// (or produced NaN) stays in the state.
int advance(Handle *H, double dt, int nsteps) {
  if (!H->state_set) return set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (nsteps < 0 || !(std::isfinite(dt))) return set_error(H, IMODEL_SWM_EINVAL, "bad dt or nsteps");
  if (nsteps == 0) return IMODEL_SWM_OK;
  if (!H->learned_active) return launch_steps(H, dt, nsteps);
  for (int done = 0; done < nsteps;) {
    const int k = std::min(kGuardSteps, nsteps - done);
    if (!H->learned_active) return launch_steps(H, dt, nsteps - done);
    int rc = save_checkpoint(H);
    if (rc) return rc;
    if ((rc = launch_steps(H, dt, k))) return rc;
    bool tripped = false;
    if ((rc = learned_guard(H, &tripped, k))) return rc;
    if (tripped) {
      if ((rc = roll_back(H))) return rc;
      if ((rc = launch_steps(H, dt, k))) return rc;
    }
    done += k;
  }
  return IMODEL_SWM_OK;
}

// imodel_swm_step with host arrays.  With the learned correction on and at
// most one guard interval of steps, the energy check runs on the second
// stream while the state is written back, and one synchronisation serves
// the check and the flags; a failed check rolls the interval back, steps it
// with the plain scheme and writes the state back again.
int step_host(Handle *H, double *h, double *u, double dt, int nsteps) {
  int rc = load_state(H, h, u, false);
  if (rc) return rc;
  const bool overlap = H->learned_active && H->te_ref_set && H->side && nsteps > 0 &&
                       nsteps <= kGuardSteps && std::isfinite(dt);
  if (!overlap) {
    if ((rc = advance(H, dt, nsteps)) || (rc = store_state(H, h, u))) return rc;
    return check_flags(H);
  }
  if ((rc = save_checkpoint(H)) || (rc = launch_steps(H, dt, nsteps))) return rc;
  CK(cudaEventRecord(H->ev_steps, H->stream));
  CK(cudaStreamWaitEvent(H->side, H->ev_steps, 0));
  if ((rc = enqueue_energy(H, H->side))) return rc;
  CK(cudaEventRecord(H->ev_side, H->side));
  if ((rc = store_state(H, h, u))) return rc;
  CK(cudaStreamWaitEvent(H->stream, H->ev_side, 0));
  int f = 0;
  if ((rc = read_flags(H, &f))) return rc;
  const double te = H->h_result[Q_PE] + H->h_result[Q_KE];
  bool trip = guard_decide(H, te, H->h_result[Q_UMAX]);
  if (!trip && (rc = error_proxy(H, nsteps, &trip))) return rc;
  if (!trip) return flags_status(H, f);
  if ((rc = roll_back(H)) || (rc = launch_steps(H, dt, nsteps)) ||
      (rc = store_state(H, h, u)))
    return rc;
  return check_flags(H);
}

// the guard's bounds and the error proxy's buffer (FP32 learned handles)
int setup_guard(Handle *H, const imodel_swm_opts *o, int ne) {
  if (!std::isfinite(o->drift_bound) || o->drift_bound < 0 || !std::isfinite(o->error_bound) ||
      o->error_bound < 0)
    return set_error(H, IMODEL_SWM_EINVAL, "drift_bound and error_bound must be finite and >= 0");
  H->drift_bound = o->drift_bound > 0 ? o->drift_bound : 1e-3;
  H->error_bound = o->error_bound > 0 ? o->error_bound : 0.25;
  return dalloc(H, &H->proxy_u, 2 * static_cast<size_t>(ne));
}

int setup_learned(Handle *H, const imodel_swm_mesh *m, const Layout &L, const imodel_swm_opts *o) {
  if (H->precision != IMODEL_SWM_FP32)
    return set_error(H, IMODEL_SWM_EINVAL, "the learned correction needs the FP32 path");
  if (!o->mlp_weights || o->mlp_bytes != static_cast<size_t>(IMODEL_MLP_NPARAM) * sizeof(float))
    return set_error(H, IMODEL_SWM_EINVAL, "mlp_weights must hold 5825 FP32 parameters");
  LearnedLayout LL;
  std::string msg = build_learned_layout(*m, L, LL);
  if (!msg.empty()) return set_error(H, IMODEL_SWM_EINVAL, msg);
  int rc;
  if ((rc = upload(H, LL.blocks, &H->learned.blocks)) ||
      (rc = dalloc(H, &H->learned.corr, static_cast<size_t>(L.ne))) ||
      (rc = dalloc(H, &H->ck_h, static_cast<size_t>(L.nv))) ||
      (rc = dalloc(H, &H->ck_u, static_cast<size_t>(L.ne))))
    return rc;
  CK(cudaStreamCreateWithFlags(&H->side, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&H->ev_steps, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&H->ev_side, cudaEventDisableTiming));
  rc = learned_prepare(static_cast<const float *>(o->mlp_weights), &H->learned, H->stream);
  if (H->learned.p) H->allocs.push_back(H->learned.p);
  if (H->learned.img) H->allocs.push_back(H->learned.img);
  if (rc) return set_error(H, rc, "learned correction set-up failed");
  if ((rc = setup_guard(H, o, L.ne))) return rc;
  H->learned_on = H->learned_active = true;
  H->learned_mode = 1;
  H->W32.learned = &H->learned;
  H->W32.tune.variant = 1;
  return IMODEL_SWM_OK;
}

// Learned TRSK weights (opts.learned = 2): the network corrects every kite
// fraction from local geometry once (imodel_gb300/learned_weights.py); the
// weights are rebuilt from the corrected fractions.  On success *m2 views
// the caller's mesh with H->kite_hxtr / H->kite_trskw in place of
// hx_hxtr_area / hx_trskw.
int learned_weights(Handle *H, const imodel_swm_mesh *m, const imodel_swm_opts *o,
                    imodel_swm_mesh *m2) {
  if (!o->mlp_weights || o->mlp_bytes != static_cast<size_t>(IMODEL_MLP_NPARAM) * sizeof(float))
    return set_error(H, IMODEL_SWM_EINVAL, "mlp_weights must hold 5825 FP32 parameters");
  KiteInputs K;
  std::string msg = build_kite_inputs(*m, K);
  if (!msg.empty()) return set_error(H, IMODEL_SWM_EINVAL, msg);
  const int64_t n = static_cast<int64_t>(K.cell.size());
  imodel::HVec<float> y;  // every output written by the network
  y.resize(static_cast<size_t>(n));
  void *net = nullptr;
  int rc = imodel_mlp_create(H->device, &net);
  if (!rc) rc = imodel_mlp_set_params(net, static_cast<const float *>(o->mlp_weights),
                                      IMODEL_MLP_NPARAM);
  if (!rc) rc = imodel_mlp_forward(net, K.x.data(), n, y.data());
  if (rc) {
    const char *e = net ? imodel_mlp_last_error(net) : "";
    std::string what = std::string("learned weights: network evaluation failed: ") + (e ? e : "");
    if (net) imodel_mlp_destroy(net);
    return set_error(H, rc, what);
  }
  imodel_mlp_destroy(net);
  apply_kite_outputs(*m, K, y.data(), H->kite_hxtr, H->kite_trskw);
  *m2 = *m;
  m2->hx_hxtr_area = H->kite_hxtr.data();
  m2->hx_trskw = H->kite_trskw.data();
  return IMODEL_SWM_OK;
}

int create(Handle *H, const imodel_swm_mesh *m, const imodel_swm_opts *o) {
  H->precision = o ? o->precision : IMODEL_SWM_FP64;
  H->testcase = o ? o->testcase : 2;
  H->device = o ? o->device : 0;
  if (H->precision != IMODEL_SWM_FP64 && H->precision != IMODEL_SWM_FP32)
    return set_error(H, IMODEL_SWM_EINVAL, "precision must be IMODEL_SWM_FP64 or IMODEL_SWM_FP32");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return set_error(H, IMODEL_SWM_ENODEV, "no CUDA device");
  if (H->device < 0 || H->device >= ndev) return set_error(H, IMODEL_SWM_EINVAL, "bad device ordinal");
  CK(cudaSetDevice(H->device));
  const int scheme = o ? o->scheme : IMODEL_SWM_TRSK10;
  if (scheme < IMODEL_SWM_TRSK10 || scheme > IMODEL_SWM_DTRED)
    return set_error(H, IMODEL_SWM_EINVAL, "unknown scheme");
  const int fsphere = o ? o->fsphere : 0;
  const double fcte = o ? o->fcte : 0.0;
  if (fsphere != 0 && fsphere != 2)
    return set_error(H, IMODEL_SWM_EINVAL, "fsphere must be 0 (f = 2 Omega sin lat) or 2 (f = fcte)");
  if (fsphere == 2 && !std::isfinite(fcte)) return set_error(H, IMODEL_SWM_EINVAL, "fcte must be finite");
  const int lmode = o ? o->learned : 0;
  if (lmode < 0 || lmode > 2)
    return set_error(H, IMODEL_SWM_EINVAL,
                     "learned must be 0, 1 (per-step network) or 2 (learned weights)");
  if (lmode != 0 && scheme != IMODEL_SWM_TRSK10)
    return set_error(H, IMODEL_SWM_EINVAL, "the learned corrections are built on trsk10 only");
  imodel_swm_mesh mk{};
  const imodel_swm_mesh *mesh = m;
  if (lmode == 2) {
    const int rc0 = learned_weights(H, m, o, &mk);
    if (rc0) return rc0;
    mesh = &mk;
    H->learned_mode = 2;
  }
  Layout L;
  std::string msg = build_layout(*mesh, o ? o->bt : nullptr, L, scheme, fsphere, fcte);
  if (!msg.empty()) return set_error(H, IMODEL_SWM_EINVAL, msg);
  H->nv = L.nv;
  H->ne = L.ne;
  H->nt = L.nt;
  H->h_areag.assign(m->hx_areag, m->hx_areag + L.nv);
  for (int i = 0; i < L.nv; ++i) H->area_cells += L.c_areag[i];
  for (int e = 0; e < L.ne; ++e) H->area_edges += L.e_area[e];
  if (o && H->precision == IMODEL_SWM_FP32 && o->h_ref != 0.0) {
    H->W32.h_ref = static_cast<float>(o->h_ref);
    H->h_ref = static_cast<double>(H->W32.h_ref);
    H->href_fixed = true;
  }
  CK(cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking));
  DevMesh &M = H->M;
  M.nv = L.nv;
  M.ne = L.ne;
  M.nt = L.nt;
  M.erad = L.erad;
  M.grav = L.grav;
  int rc = 0;
  std::vector<float> bt32(L.c_bt.size());
  for (size_t i = 0; i < bt32.size(); ++i) bt32[i] = static_cast<float>(L.c_bt[i]);
  if ((rc = upload(H, L.c_nnb, &M.c_nnb)) || (rc = upload(H, L.c_ed, &M.c_ed)) ||
      (rc = upload(H, L.c_sd, &M.c_sd)) || (rc = upload(H, L.c_areag, &M.c_areag)) ||
      (rc = upload(H, L.c_cellarea, &M.c_cellarea)) || (rc = upload(H, L.c_bt, &M.c_bt)) ||
      (rc = upload(H, L.e_v, &M.e_v)) || (rc = upload(H, L.e_sh, &M.e_sh)) ||
      (rc = upload(H, L.e_leng, &M.e_leng)) || (rc = upload(H, L.e_dleng, &M.e_dleng)) ||
      (rc = upload(H, L.e_kew, &M.e_kew)) || (rc = upload(H, L.e_area, &M.e_area)) ||
      (rc = upload(H, L.e_nst, &M.e_nst)) || (rc = upload(H, L.e_stk, &M.e_stk)) ||
      (rc = upload(H, L.e_stw, &M.e_stw)) || (rc = upload(H, L.t_ed, &M.t_ed)) ||
      (rc = upload(H, L.t_v, &M.t_v)) || (rc = upload(H, L.t_lt, &M.t_lt)) ||
      (rc = upload(H, L.t_kite, &M.t_kite)) || (rc = upload(H, L.t_areag, &M.t_areag)) ||
      (rc = upload(H, L.t_f, &M.t_f)) || (rc = upload(H, L.e_sgtg, &M.e_sgtg)) ||
      (rc = upload(H, L.e_gtg32, &M.e_gtg32)))
    return rc;
  if (H->precision == IMODEL_SWM_FP32) {
    if ((rc = upload(H, L.c_div32, &M.c_div32)) || (rc = upload(H, L.c_kew32, &M.c_kew32)) ||
        (rc = upload(H, bt32, &M.c_bt32)) || (rc = upload(H, L.e_grad32, &M.e_grad32)) ||
        (rc = upload(H, L.e_stc32, &M.e_stc32)) || (rc = upload(H, L.t_f32, &M.t_f32)) ||
        (rc = upload(H, L.c_nb, &M.c_nb)) || (rc = upload(H, L.c_tr, &M.c_tr)) ||
        (rc = upload(H, L.c_R32, &M.c_R32)) || (rc = upload(H, L.c_dg32, &M.c_dg32)) ||
        (rc = upload(H, L.c_inva32, &M.c_inva32)) || (rc = upload(H, L.c_meta, &M.c_meta)) ||
        (rc = upload(H, L.e_vs, &M.e_vs)))
      return rc;
    const int32_t *ra = nullptr, *rb = nullptr, *rc32 = nullptr;
    if ((rc = upload(H, L.t_recA, &ra)) || (rc = upload(H, L.t_recB, &rb)) ||
        (rc = upload(H, L.t_recC, &rc32)))
      return rc;
    M.t_recA = reinterpret_cast<const int4 *>(ra);
    M.t_recB = reinterpret_cast<const int4 *>(rb);
    M.t_recC = reinterpret_cast<const float4 *>(rc32);
    std::vector<float> c_area32(L.c_areag.begin(), L.c_areag.end());
    std::vector<float> e_area32(L.e_area.begin(), L.e_area.end());
    if ((rc = upload(H, c_area32, &M.c_area32)) || (rc = upload(H, e_area32, &M.e_area32)))
      return rc;
    const int32_t *pk = nullptr;
    const float *kd = nullptr;
    const uint32_t *vs2 = nullptr;
    if ((rc = upload(H, L.c_pk, &pk)) || (rc = upload(H, L.c_kd, &kd)) ||
        (rc = upload(H, L.e_vs2, &vs2)))
      return rc;
    // cudaMalloc returns 256-byte aligned memory: safe to view as int4/float2/uint2
    M.c_pk = reinterpret_cast<const int4 *>(pk);
    M.c_kd = reinterpret_cast<const float2 *>(kd);
    M.e_vs2 = reinterpret_cast<const uint2 *>(vs2);
    const uint32_t *ta = nullptr;
    const int32_t *twb = nullptr;
    const float *tb = nullptr, *tc = nullptr;
    if ((rc = upload(H, L.t_c16A, &ta)) || (rc = upload(H, L.t_c16B, &tb)) ||
        (rc = upload(H, L.t_c16C, &tc)) || (rc = upload(H, L.t_wb, &twb)))
      return rc;
    M.t_c16A = reinterpret_cast<const uint4 *>(ta);
    M.t_c16B = reinterpret_cast<const float4 *>(tb);
    M.t_c16C = reinterpret_cast<const float2 *>(tc);
    M.t_wb = reinterpret_cast<const int2 *>(twb);
  }
  const int32_t *cn2o = nullptr, *en2o = nullptr;
  if ((rc = upload(H, L.cell_n2o, &cn2o)) || (rc = upload(H, L.edge_n2o, &en2o))) return rc;
  H->dif_ok = m->ed_nr != nullptr;
  // the APVM reconstructions (FP64 step) read the edge, triangle and cell points
  if (H->precision == IMODEL_SWM_FP64 && !L.t_c.empty()) {
    if ((rc = upload(H, L.e_c, &M.e_c)) || (rc = upload(H, L.t_c, &M.t_c)) ||
        (rc = upload(H, L.c_p, &M.c_p)))
      return rc;
  }
  // the other method wrappers' geometry (empty vectors upload as NULL)
  if (H->precision == IMODEL_SWM_FP32 &&
      ((rc = upload(H, L.c_C32, &M.c_C32)) || (rc = upload(H, L.c_gout, &M.c_gout)) ||
       (rc = upload(H, L.c_qw32, &M.c_qw32)) || (rc = upload(H, L.t_dpa32, &M.t_dpa32)) ||
       (rc = upload(H, L.t_dopp, &M.t_dopp)) || (rc = upload(H, L.e_nr32, &M.e_nr32)) ||
       (rc = upload(H, L.e_dw32, &M.e_dw32))))
    return rc;
  if ((rc = upload(H, L.t_bary, &M.t_bary)) || (rc = upload(H, L.e_dist, &M.e_dist)) ||
      (rc = upload(H, L.t_edarea, &M.t_edarea)) || (rc = upload(H, L.e_nr, &M.e_nr)) ||
      (rc = upload(H, L.e_stq, &M.e_stq)))
    return rc;
  if (H->precision == IMODEL_SWM_FP32 &&
      ((rc = upload(H, L.e_qw32, &M.e_qw32)) || (rc = upload(H, L.e_dtc32, &M.e_dtc32))))
    return rc;
  if (H->precision == IMODEL_SWM_FP32 && !L.t_apw32.empty()) {
    if ((rc = upload(H, L.t_apw32, &M.t_apw32)) || (rc = upload(H, L.t_cc32, &M.t_cc32)) ||
        (rc = upload(H, L.c_apw32, &M.c_apw32)) || (rc = upload(H, L.c_p32, &M.c_p32)))
      return rc;
  }
  H->d_cell_n2o = const_cast<int32_t *>(cn2o);
  H->d_edge_n2o = const_cast<int32_t *>(en2o);
  const int32_t *co2n = nullptr, *eo2n = nullptr;
  if ((rc = upload(H, L.cell_o2n, &co2n)) || (rc = upload(H, L.edge_o2n, &eo2n))) return rc;
  H->d_cell_o2n = const_cast<int32_t *>(co2n);
  H->d_edge_o2n = const_cast<int32_t *>(eo2n);
  {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault,
                                         &qr) == cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      H->range_attr = reinterpret_cast<CUresult (*)(void *, CUpointer_attribute, CUdeviceptr)>(fn);
    cudaGetLastError();
  }
  if ((rc = dalloc(H, &H->d_stage_h, L.nv)) || (rc = dalloc(H, &H->d_stage_u, L.ne)) ||
      (rc = dalloc(H, &H->d_ref_h, L.nv)) || (rc = dalloc(H, &H->d_ref_u, L.ne)) ||
      (rc = dalloc(H, &H->d_scratch, static_cast<size_t>(2) * kRedBlocks * 16)) ||
      (rc = dalloc(H, &H->d_result, 16)) || (rc = dalloc(H, &H->d_flags, 1)))
    return rc;
  CK(cudaMallocHost(&H->h_flags, sizeof(int)));
  CK(cudaMallocHost(&H->h_result, 16 * sizeof(double)));
  if (H->precision == IMODEL_SWM_FP64) {
    if (o && o->learned == 1)
      return set_error(H, IMODEL_SWM_EINVAL, "the per-step learned correction needs the FP32 path");
    if ((rc = alloc_work(H, H->W64))) return rc;
    H->W64.scheme = scheme;
    if (scheme == IMODEL_SWM_GASS18 &&
        ((rc = dalloc(H, &H->W64.eta_t, L.nt)) || (rc = dalloc(H, &H->W64.h_trs, L.nt))))
      return rc;
    if (scheme == IMODEL_SWM_DTRED && (rc = dalloc(H, &H->W64.vhq, 3 * static_cast<size_t>(L.nt))))
      return rc;
  } else {
    const float keep = H->W32.h_ref;
    if ((rc = alloc_work(H, H->W32))) return rc;
    H->W32.h_ref = keep;
    if ((rc = dalloc(H, &H->W32.zflux, static_cast<size_t>(kMaxNb) * L.nv))) return rc;
    // the method wrappers run in every variant (the cell-centred ones with
    // their coefficients by cell or, for dtred, by triangle)
    H->W32.scheme = scheme;
    H->v0_only = scheme == IMODEL_SWM_GASS18 && !L.gass_cells;
    if (H->v0_only) H->W32.tune.variant = 0;
    if (scheme == IMODEL_SWM_GASS18 && (rc = dalloc(H, &H->W32.h_trs, L.nt))) return rc;
    if (scheme == IMODEL_SWM_DTRED && (rc = dalloc(H, &H->W32.vhq, 3 * static_cast<size_t>(L.nt))))
      return rc;
    if (o && o->learned == 1 && (rc = setup_learned(H, m, L, o))) return rc;
  }
  if (H->learned_mode == 2) {
    H->w_learned = {M.e_stw, M.e_stc32, M.c_R32, M.c_pk};
    if (H->precision == IMODEL_SWM_FP32) {
      // the guard's fallback: the plain scheme's weight-dependent arrays
      WeightArrays Lp;
      msg = build_weight_arrays(*m, L, Lp);
      if (!msg.empty()) return set_error(H, IMODEL_SWM_EINVAL, msg);
      const int32_t *pk = nullptr;
      if ((rc = upload(H, Lp.e_stw, &H->w_plain.e_stw)) ||
          (rc = upload(H, Lp.e_stc32, &H->w_plain.e_stc32)) ||
          (rc = upload(H, Lp.c_R32, &H->w_plain.c_R32)) || (rc = upload(H, Lp.c_pk, &pk)))
        return rc;
      H->w_plain.c_pk = reinterpret_cast<const int4 *>(pk);
      if ((rc = dalloc(H, &H->ck_h, static_cast<size_t>(L.nv))) ||
          (rc = dalloc(H, &H->ck_u, static_cast<size_t>(L.ne))))
        return rc;
      CK(cudaStreamCreateWithFlags(&H->side, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&H->ev_steps, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&H->ev_side, cudaEventDisableTiming));
      if ((rc = setup_guard(H, o, L.ne))) return rc;
      H->learned_on = H->learned_active = true;
    }
  }
  CK(cudaDeviceSynchronize());
  return IMODEL_SWM_OK;
}

void destroy(Handle *H) {
  if (!H) return;
  if (H->graph) cudaGraphExecDestroy(H->graph);
  if (H->stream) cudaStreamSynchronize(H->stream);
  for (void *p : H->allocs) cudaFree(p);
  if (H->h_flags) cudaFreeHost(H->h_flags);
  if (H->h_result) cudaFreeHost(H->h_result);
  if (H->side) cudaStreamSynchronize(H->side);
  if (H->ev_steps) cudaEventDestroy(H->ev_steps);
  if (H->ev_side) cudaEventDestroy(H->ev_side);
  if (H->side) cudaStreamDestroy(H->side);
  if (H->stream) cudaStreamDestroy(H->stream);
  delete H;
}

// The coefficients and work arrays of the (hyper)diffusion terms: constant
// k2 / k4, or, with kf2 / kf4 (host, reference cell order) not NULL, those
// per-cell fields (the "align" and "diam" branches).
template <class T>
int setup_diffusion(Handle *H, Work<T> &W, double k2, double k4, const double *kf2,
                    const double *kf4) {
  Diffusion<T> &D = W.dif;
  // the terms stay off until every buffer and coefficient is in place: a
  // failure below leaves the handle stepping without diffusion
  D.on = false;
  const bool k2on = k2 > 0 || kf2, k4on = k4 > 0 || kf4;
  if (!k2on && !k4on) {
    D.k2 = D.k4 = false;
    return IMODEL_SWM_OK;
  }
  int rc;
  // each buffer on its own, so that a call after a failed one completes the set
  if ((!D.kt && (rc = dalloc(H, &D.kt, H->nt))) || (!D.kcv && (rc = dalloc(H, &D.kcv, H->nv))) ||
      (!D.coefdiv && (rc = dalloc(H, &D.coefdiv, H->nv))) ||
      (!D.coefvort && (rc = dalloc(H, &D.coefvort, H->nt))) ||
      (!D.lap && (rc = dalloc(H, &D.lap, H->ne))) || (!D.lap2 && (rc = dalloc(H, &D.lap2, H->ne))))
    return rc;
  double *kt64 = nullptr, *kc64 = nullptr;
  float *kt32 = nullptr, *kc32 = nullptr;
  if (sizeof(T) == sizeof(double)) {
    kt64 = reinterpret_cast<double *>(D.kt);
    kc64 = reinterpret_cast<double *>(D.kcv);
  } else {
    if ((!H->d_kt64 && (rc = dalloc(H, &H->d_kt64, H->nt))) ||
        (!H->d_kc64 && (rc = dalloc(H, &H->d_kc64, H->nv))))
      return rc;
    kt64 = H->d_kt64;
    kc64 = H->d_kc64;
    kt32 = reinterpret_cast<float *>(D.kt);
    kc32 = reinterpret_cast<float *>(D.kcv);
  }
  // swm.f90:169-205: K at the cells, hx2tr(K) at the triangles;
  // hyperdiffusion applies the Laplacian twice with sqrt(K4) and
  // sqrt(hx2tr(K4)), and then also replaces the Laplacian's coefficients
  const double *kf = k4on ? kf4 : kf2;
  double *kf_dev = nullptr;
  if (kf) {
    const size_t nv = static_cast<size_t>(H->nv);
    if (!H->d_kf && (rc = dalloc(H, &H->d_kf, 2 * nv))) return rc;
    CK(cudaMemcpyAsync(H->d_kf, kf, nv * sizeof(double), cudaMemcpyHostToDevice, H->stream));
    launch_gather_in(H->nv, H->d_cell_n2o, H->d_kf, H->d_kf + nv, 0.0, H->stream);
    kf_dev = H->d_kf + nv;
  }
  launch_dif_coefs(H->M, kf_dev, k4on ? k4 : k2, k4on, kc64, kc32, kt64, kt32, H->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(H->stream));
  D.k2 = k2on;
  D.k4 = k4on;
  D.on = true;
  return IMODEL_SWM_OK;
}
// the anticipated potential vorticity method (apvm, swm_operators.f90:
// 1465-1543) with parameter pvspar and the run's time step dt: the
// tendency reads dt from the module (swm.f90:2558), not from the stage
template <class T>
int setup_apvm(Handle *H, Work<T> &W, double pvspar, double dt) {
  Apvm<T> &A = W.apvm;
  // off until all three buffers exist: a failed allocation leaves the handle
  // stepping without APVM instead of launching through a null buffer
  A.on = false;
  if (!(pvspar > 0)) return IMODEL_SWM_OK;
  int rc;
  if ((!A.qg && (rc = dalloc(H, &A.qg, 3 * static_cast<size_t>(H->nt)))) ||
      (!A.vhx && (rc = dalloc(H, &A.vhx, 3 * static_cast<size_t>(H->nv)))) ||
      (!A.qge && (rc = dalloc(H, &A.qge, static_cast<size_t>(H->ne)))))
    return rc;
  A.coef = static_cast<T>(pvspar * dt);
  A.on = true;
  return IMODEL_SWM_OK;
}
}  // namespace
}  // namespace imodel

using imodel::Handle;

extern "C" {

int imodel_swm_create(const imodel_swm_mesh *m, const imodel_swm_opts *o, void **handle) {
  if (!handle) return IMODEL_SWM_EINVAL;
  *handle = nullptr;
  Handle *H = new (std::nothrow) Handle();
  if (!H) return IMODEL_SWM_ENOMEM;
  if (!m) {
    *handle = H;
    H->err = "mesh is NULL";
    return IMODEL_SWM_EINVAL;
  }
  int rc;
  try {
    rc = imodel::create(H, m, o);
  } catch (const std::bad_alloc &) {
    rc = IMODEL_SWM_ENOMEM;
    H->err = "host allocation failed";
  }
  // the handle is returned even on failure so that last_error can be read;
  // it must still be destroyed
  *handle = H;
  return rc;
}

int imodel_swm_step(void *handle, double *h_io, double *u_io, double dt, int32_t nsteps) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !h_io || !u_io) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  return imodel::step_host(H, h_io, u_io, dt, nsteps);
}

int imodel_swm_set_state(void *handle, const double *h, const double *u) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !h || !u) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc = imodel::load_state(H, h, u, true);
  if (rc) return rc;
  if (cudaStreamSynchronize(H->stream) != cudaSuccess)
    return imodel::set_error(H, IMODEL_SWM_ECUDA, "stream synchronize failed");
  return IMODEL_SWM_OK;
}

int imodel_swm_get_state(void *handle, double *h, double *u) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !h || !u) return IMODEL_SWM_EINVAL;
  if (!H->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc = imodel::store_state(H, h, u);
  if (rc) return rc;
  return imodel::check_flags(H);
}

int imodel_swm_advance(void *handle, double dt, int32_t nsteps) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return IMODEL_SWM_EINVAL;
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc = imodel::advance(H, dt, nsteps);
  if (rc) return rc;
  return imodel::check_flags(H);
}

int imodel_swm_tendency(void *handle, const double *h, const double *u, double *masseq,
                        double *momeq) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !h || !u || !masseq || !momeq) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  if (H->precision == IMODEL_SWM_FP32 && !H->href_fixed) {
    double s = 0.0, a = 0.0;
    for (int i = 0; i < H->nv; ++i) {
      a += H->h_areag[i];
      s += H->h_areag[i] * h[i];
    }
    H->W32.h_ref = static_cast<float>(s / a);
    H->h_ref = static_cast<double>(H->W32.h_ref);
    H->href_fixed = true;
  }
  cudaError_t e;
  e = cudaMemcpyAsync(H->d_stage_h, h, sizeof(double) * H->nv, cudaMemcpyHostToDevice, H->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->d_stage_u, u, sizeof(double) * H->ne, cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  // the tendency input becomes the "last stage input" the diagnostics use
  if (H->precision == IMODEL_SWM_FP64) {
    auto &W = H->W64;
    imodel::launch_gather_in(H->nv, H->d_cell_n2o, H->d_stage_h, W.ya_h, 0.0, H->stream);
    imodel::launch_gather_in(H->ne, H->d_edge_n2o, H->d_stage_u, W.ya_u, 0.0, H->stream);
    imodel::launch_stage64(H->M, W, W.ya_h, W.ya_u, nullptr, nullptr, -1, 0.0, H->stream);
    imodel::launch_scatter_out(H->nv, H->d_cell_n2o, W.tend_h, H->d_stage_h, 0.0, nullptr, H->stream);
    imodel::launch_scatter_out(H->ne, H->d_edge_n2o, W.tend_u, H->d_stage_u, 0.0, nullptr, H->stream);
  } else {
    auto &W = H->W32;
    imodel::launch_gather_in32(H->nv, H->d_cell_n2o, H->d_stage_h, W.ya_h, H->h_ref, H->stream);
    imodel::launch_gather_in32(H->ne, H->d_edge_n2o, H->d_stage_u, W.ya_u, 0.0, H->stream);
    imodel::launch_stage32(H->M, W, W.ya_h, W.ya_u, nullptr, nullptr, -1, 0.0f, H->stream);
    imodel::launch_scatter_out32(H->nv, H->d_cell_n2o, W.tend_h, H->d_stage_h, 0.0, nullptr, H->stream);
    imodel::launch_scatter_out32(H->ne, H->d_edge_n2o, W.tend_u, H->d_stage_u, 0.0, nullptr, H->stream);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(masseq, H->d_stage_h, sizeof(double) * H->nv, cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(momeq, H->d_stage_u, sizeof(double) * H->ne, cudaMemcpyDeviceToHost, H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  return imodel::check_flags(H);
}

int imodel_swm_diagnostics(void *handle, imodel_swm_diag *out) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !out) return IMODEL_SWM_EINVAL;
  if (!H->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  if (H->precision == IMODEL_SWM_FP64) {
    auto &W = H->W64;
    imodel::launch_diag<double>(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, H->d_scratch,
                                H->d_result, H->stream);
  } else {
    auto &W = H->W32;
    imodel::launch_diag<float>(H->M, W, W.yn_h, W.yn_u, W.ya_h, W.ya_u, H->d_scratch,
                               H->d_result, H->stream);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->h_result, H->d_result, sizeof(double) * imodel::kDiagQ,
                        cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  const double *r = H->h_result;
  const double g = H->M.grav;
  const double A = r[imodel::Q_AREA];
  std::memset(out, 0, sizeof(*out));
  out->mass = r[imodel::Q_AH] / A;
  out->penergy = r[imodel::Q_PE];
  out->kenergy = r[imodel::Q_KE];
  out->tenergy = out->penergy + out->kenergy;
  const double mh = r[imodel::Q_AHB] / A;
  const double unavail = 0.5 * g * (mh * mh * A - r[imodel::Q_AB2]);
  out->availenergy = out->tenergy - unavail;
  out->pot_enstrophy = r[imodel::Q_ENS];
  out->rms_div = std::sqrt(r[imodel::Q_ADIV2] / A);
  out->max_div = r[imodel::Q_MAXDIV];
  out->nan_found = r[imodel::Q_NAN] != 0.0 ? 1 : 0;
  // an FP64 handle with learned weights has no guard: they stay applied
  out->learned_active =
      (H->learned_active || (H->learned_mode == 2 && !H->learned_on)) ? 1 : 0;
  return IMODEL_SWM_OK;
}

int imodel_swm_errors(void *handle, const double *h_ref, const double *u_ref, double out[6]) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !h_ref || !u_ref || !out) return IMODEL_SWM_EINVAL;
  if (!H->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  cudaError_t e;
  e = cudaMemcpyAsync(H->d_stage_h, h_ref, sizeof(double) * H->nv, cudaMemcpyHostToDevice, H->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->d_stage_u, u_ref, sizeof(double) * H->ne, cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  imodel::launch_gather_in(H->nv, H->d_cell_n2o, H->d_stage_h, H->d_ref_h, 0.0, H->stream);
  imodel::launch_gather_in(H->ne, H->d_edge_n2o, H->d_stage_u, H->d_ref_u, 0.0, H->stream);
  if (H->precision == IMODEL_SWM_FP64)
    imodel::launch_errors<double>(H->M, H->W64.yn_h, H->W64.yn_u, 0.0, H->d_ref_h, H->d_ref_u,
                                  H->d_scratch, H->d_result, H->stream);
  else
    imodel::launch_errors<float>(H->M, H->W32.yn_h, H->W32.yn_u, H->h_ref, H->d_ref_h,
                                 H->d_ref_u, H->d_scratch, H->d_result, H->stream);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->h_result, H->d_result, sizeof(double) * 8, cudaMemcpyDeviceToHost,
                        H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  const double *r = H->h_result;
  // h: r[0] sum A dif^2, r[1] sum A ref^2, r[2] max|dif|, r[3] max|ref|
  for (int f = 0; f < 2; ++f) {
    const double *q = r + 4 * f;
    const double area = f == 0 ? H->area_cells : H->area_edges;
    out[3 * f + 0] = q[3] > 0 ? q[2] / q[3] : q[2];
    out[3 * f + 1] = q[1] > 0 ? std::sqrt(q[0] / area) / std::sqrt(q[1] / area)
                              : std::sqrt(q[0] / area);
    out[3 * f + 2] = q[2];
  }
  return IMODEL_SWM_OK;
}

int imodel_swm_trsk_tangent(void *handle, const double *u, double *utg) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !u || !utg) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  cudaError_t e = cudaMemcpyAsync(H->d_stage_u, u, sizeof(double) * H->ne,
                                  cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  imodel::launch_gather_in(H->ne, H->d_edge_n2o, H->d_stage_u, H->d_ref_u, 0.0, H->stream);
  imodel::launch_trsk_tangent(H->M, H->d_ref_u, H->d_stage_u, H->stream);
  // d_stage_u now holds utg in device order; scatter it through d_ref_u
  imodel::launch_scatter_out(H->ne, H->d_edge_n2o, H->d_stage_u, H->d_ref_u, 0.0, nullptr,
                             H->stream);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(utg, H->d_ref_u, sizeof(double) * H->ne, cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  return IMODEL_SWM_OK;
}

int imodel_swm_profile(void *handle, double dt, int32_t nsteps, double avg_ms[4]) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !avg_ms || nsteps <= 0) return IMODEL_SWM_EINVAL;
  if (!H->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  cudaEvent_t ev[5];
  for (int k = 0; k < 5; ++k)
    if (cudaEventCreate(&ev[k]) != cudaSuccess)
      return imodel::set_error(H, IMODEL_SWM_ECUDA, "cudaEventCreate failed");
  double sum[4] = {0, 0, 0, 0};
  cudaError_t e = cudaSuccess;
  for (int step = 0; step < nsteps && e == cudaSuccess; ++step) {
    for (int st = 0; st < 4 && e == cudaSuccess; ++st) {
      if (H->precision == IMODEL_SWM_FP64) {
        auto &W = H->W64;
        const double *hi[4] = {W.yn_h, W.ya_h, W.yb_h, W.ya_h};
        const double *ui[4] = {W.yn_u, W.ya_u, W.yb_u, W.ya_u};
        double *ho[4] = {W.ya_h, W.yb_h, W.ya_h, W.yn_h};
        double *uo[4] = {W.ya_u, W.yb_u, W.ya_u, W.yn_u};
        imodel::launch_stage64(H->M, W, hi[st], ui[st], ho[st], uo[st], st, dt, H->stream, ev);
      } else {
        auto &W = H->W32;
        const float *hi[4] = {W.yn_h, W.ya_h, W.yb_h, W.ya_h};
        const float *ui[4] = {W.yn_u, W.ya_u, W.yb_u, W.ya_u};
        float *ho[4] = {W.ya_h, W.yb_h, W.ya_h, W.yn_h};
        float *uo[4] = {W.ya_u, W.yb_u, W.ya_u, W.yn_u};
        imodel::launch_stage32(H->M, W, hi[st], ui[st], ho[st], uo[st], st,
                               static_cast<float>(dt), H->stream, ev);
      }
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
      for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
        sum[k] += ms;
      }
    }
  }
  for (int k = 0; k < 5; ++k) cudaEventDestroy(ev[k]);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  for (int k = 0; k < 4; ++k) avg_ms[k] = sum[k] / (4.0 * nsteps);
  return imodel::check_flags(H);
}

int imodel_swm_autotune(void *handle, double dt, int32_t nsteps, int32_t choice[6]) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !choice || nsteps <= 0) return IMODEL_SWM_EINVAL;
  if (!H->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  if (H->precision == IMODEL_SWM_FP64) {
    // the FP64 path has one variant; its launch shape is fixed
    choice[0] = 0;
    choice[1] = choice[2] = choice[3] = choice[4] = 256;
    choice[5] = 0;
    return IMODEL_SWM_OK;
  }
  auto &W = H->W32;
  const size_t bh = sizeof(float) * H->nv, bu = sizeof(float) * H->ne;
  float *save = nullptr;
  if (cudaMalloc(&save, 2 * (bh + bu)) != cudaSuccess)
    return imodel::set_error(H, IMODEL_SWM_ENOMEM, "autotune: no room to save the state");
  char *sp = reinterpret_cast<char *>(save);
  cudaError_t e = cudaSuccess;
  auto cpy = [&](void *dst, const void *src, size_t n) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, H->stream);
  };
  cpy(sp, W.yn_h, bh);
  cpy(sp + bh, W.yn_u, bu);
  cpy(sp + bh + bu, W.ya_h, bh);
  cpy(sp + 2 * bh + bu, W.ya_u, bu);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  auto trial = [&](const imodel::Tune &t) -> float {
    W.tune = t;
    if (H->graph) {
      cudaGraphExecDestroy(H->graph);
      H->graph = nullptr;
    }
    if (e != cudaSuccess || imodel::ensure_graph(H, dt)) return 1e30f;
    if ((e = cudaGraphLaunch(H->graph, H->stream)) != cudaSuccess) return 1e30f;  // warm-up
    cudaEventRecord(e0, H->stream);
    for (int k = 0; k < nsteps && e == cudaSuccess; ++k) e = cudaGraphLaunch(H->graph, H->stream);
    cudaEventRecord(e1, H->stream);
    float ms = 1e30f;
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    return e == cudaSuccess ? ms : 1e30f;
  };
  const int sizes[3] = {128, 256, 512};
  imodel::Tune best;
  float best_ms = 1e30f;
  // the learned correction is wired into the cell-centred variants only
  for (int v = H->learned_mode == 1 ? 1 : 0; v <= (H->v0_only ? 0 : 2); ++v)
    for (int b : sizes) {
      imodel::Tune t;
      t.variant = v;
      t.bs_tri = t.bs_pre = t.bs_cell = t.bs_edge = b;
      const float ms = trial(t);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  // refine the block size of each kernel with the others fixed
  int imodel::Tune::*fields[4] = {&imodel::Tune::bs_tri, &imodel::Tune::bs_pre,
                                  &imodel::Tune::bs_cell, &imodel::Tune::bs_edge};
  for (int f = 0; f < 4; ++f) {
    if (f == 1 && best.variant >= 1) continue;
    for (int b : sizes) {
      if (best.*fields[f] == b) continue;
      imodel::Tune t = best;
      t.*fields[f] = b;
      const float ms = trial(t);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  }
  // the learned-correction kernel's split of warps between gathering and
  // the epilogue
  if (H->learned_active && H->learned_mode == 1)
    for (int g = 2; g <= 4; ++g) {
      if (best.mlp_gather == g) continue;
      imodel::Tune t = best;
      t.mlp_gather = g;
      const float ms = trial(t);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  W.tune = best;
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  cpy(W.yn_h, sp, bh);
  cpy(W.yn_u, sp + bh, bu);
  cpy(W.ya_h, sp + bh + bu, bh);
  cpy(W.ya_u, sp + 2 * bh + bu, bu);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  if (e != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, cudaGetErrorString(e));
  choice[0] = best.variant;
  choice[1] = best.bs_tri;
  choice[2] = best.bs_pre;
  choice[3] = best.bs_cell;
  choice[4] = best.bs_edge;
  choice[5] = H->learned_mode == 1 ? best.mlp_gather : 0;
  return imodel::check_flags(H);
}

int imodel_swm_set_tuning(void *handle, const int32_t choice[6]) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !choice) return IMODEL_SWM_EINVAL;
  if (H->precision == IMODEL_SWM_FP64) return IMODEL_SWM_OK;
  for (int k = 1; k < 5; ++k)
    if (choice[k] != 128 && choice[k] != 256 && choice[k] != 512)
      return imodel::set_error(H, IMODEL_SWM_EINVAL, "block sizes must be 128, 256 or 512");
  if (choice[0] < 0 || choice[0] > 2)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "variant must be 0, 1 or 2");
  if (H->v0_only && choice[0] != 0)
    return imodel::set_error(H, IMODEL_SWM_EINVAL,
                             "gass18 runs with variant 0 only on this grid (its connecting edges "
                             "do not follow the cells' structure)");
  if (H->learned_mode == 1 && choice[0] == 0)
    return imodel::set_error(H, IMODEL_SWM_EINVAL,
                             "the learned correction runs with the cell-centred variants (1, 2) only");
  imodel::Tune t;
  t.variant = choice[0];
  t.bs_tri = choice[1];
  t.bs_pre = choice[2];
  t.bs_cell = choice[3];
  t.bs_edge = choice[4];
  if (H->learned_mode == 1) {
    if (choice[5] < 2 || choice[5] > 4)
      return imodel::set_error(H, IMODEL_SWM_EINVAL, "gather groups of the network: 2, 3 or 4");
    t.mlp_gather = choice[5];
  }
  H->W32.tune = t;
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  return IMODEL_SWM_OK;
}

int imodel_swm_set_diffusion(void *handle, double k2, double k4) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (!(k2 >= 0) || !(k4 >= 0) || !std::isfinite(k2) || !std::isfinite(k4))
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "diffusion coefficients must be finite and >= 0");
  if ((k2 > 0 || k4 > 0) && !H->dif_ok)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "the diffusion terms need the mesh's ed_nr");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  const int rc = H->precision == IMODEL_SWM_FP64
                     ? imodel::setup_diffusion(H, H->W64, k2, k4, nullptr, nullptr)
                     : imodel::setup_diffusion(H, H->W32, k2, k4, nullptr, nullptr);
  // the captured step no longer matches the options, whether or not the
  // set-up succeeded (a failure leaves the terms off)
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  return rc;
}

int imodel_swm_set_diffusion_fields(void *handle, const double *k2_hx, const double *k4_hx) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  for (const double *f : {k2_hx, k4_hx})
    if (f)
      for (int i = 0; i < H->nv; ++i)
        if (!(f[i] >= 0) || !std::isfinite(f[i]))
          return imodel::set_error(H, IMODEL_SWM_EINVAL,
                                   "diffusion coefficient fields must be finite and >= 0");
  if ((k2_hx || k4_hx) && !H->dif_ok)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "the diffusion terms need the mesh's ed_nr");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  const int rc = H->precision == IMODEL_SWM_FP64
                     ? imodel::setup_diffusion(H, H->W64, 0.0, 0.0, k2_hx, k4_hx)
                     : imodel::setup_diffusion(H, H->W32, 0.0, 0.0, k2_hx, k4_hx);
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  return rc;
}

int imodel_swm_learned_weights(void *handle, double *hxtr_area, double *trskw) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !hxtr_area || !trskw) return IMODEL_SWM_EINVAL;
  if (H->learned_mode != 2)
    return imodel::set_error(H, IMODEL_SWM_ESTATE, "the handle was not created with learned weights");
  std::memcpy(hxtr_area, H->kite_hxtr.data(), sizeof(double) * H->kite_hxtr.size());
  std::memcpy(trskw, H->kite_trskw.data(), sizeof(double) * H->kite_trskw.size());
  return IMODEL_SWM_OK;
}

int imodel_swm_learned_error_proxy(void *handle, double *value) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !value) return IMODEL_SWM_EINVAL;
  if (!H->learned_on || !H->proxy_u)
    return imodel::set_error(H, IMODEL_SWM_ESTATE, "the handle has no guarded learned correction");
  *value = H->last_proxy;
  return IMODEL_SWM_OK;
}

int imodel_swm_test_fail_alloc(int32_t after) {
  if (after < 0) return IMODEL_SWM_EINVAL;
  imodel::g_fail_alloc_after.store(after);
  return IMODEL_SWM_OK;
}

int imodel_swm_set_apvm(void *handle, double pvspar, double dt) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return IMODEL_SWM_EINVAL;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  if (!(pvspar >= 0) || !std::isfinite(pvspar))
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "pvspar must be finite and >= 0");
  if (pvspar > 0 && (!(dt > 0) || !std::isfinite(dt)))
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "apvm needs a finite dt > 0");
  const bool fp32 = H->precision == IMODEL_SWM_FP32;
  if (pvspar > 0 && !(fp32 ? H->M.t_apw32 != nullptr : H->M.t_c != nullptr))
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "apvm needs the mesh's ed_nr and ed_c");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  // FP32: the correction is applied in the edge pre-pass, which variants 1
  // and 2 run before their cell kernel when APVM is on
  const int rc = fp32 ? imodel::setup_apvm(H, H->W32, pvspar, dt)
                      : imodel::setup_apvm(H, H->W64, pvspar, dt);
  if (H->graph) {
    cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
  }
  return rc;
}

int imodel_swm_launch_count(void *handle, int32_t nsteps, int64_t *count) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H || !count || nsteps < 0) return IMODEL_SWM_EINVAL;
  const int fp32 = H->precision == IMODEL_SWM_FP32;
  const bool on = fp32 ? H->W32.dif.on : H->W64.dif.on;
  const bool k4 = fp32 ? H->W32.dif.k4 : H->W64.dif.k4;
  *count = static_cast<int64_t>(nsteps) * 4 *
           imodel::launches_per_stage(fp32, fp32 ? H->W32.tune.variant : 0, on, k4,
                                      fp32 ? H->W32.apvm.on : H->W64.apvm.on,
                                      fp32 ? H->W32.scheme : H->W64.scheme);
  // the learned correction adds one network launch per step while it is on
  if (fp32 && H->W32.learned) *count += nsteps;
  return IMODEL_SWM_OK;
}

const char *imodel_swm_main_kernel(void *handle) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return "";
  if (H->precision == IMODEL_SWM_FP64)
    return H->W64.scheme == IMODEL_SWM_PXT16 || H->W64.scheme == IMODEL_SWM_DTRED ? "k_edge64r"
                                                                                  : "k_edge64";
  const int v = H->W32.tune.variant;
  if (v >= 1 && H->W32.scheme == IMODEL_SWM_PXT16) return "k_cell32p";
  if (v >= 1 && H->W32.scheme == IMODEL_SWM_GASS18) return "k_cell32g";
  if (v >= 1 && H->W32.scheme == IMODEL_SWM_DTRED) return "k_cell32v2";
  return v >= 1 ? "k_cell32v2" : "k_edge32";
}

void *imodel_swm_stream(void *handle) {
  Handle *H = static_cast<Handle *>(handle);
  return H ? static_cast<void *>(H->stream) : nullptr;
}

int imodel_swm_destroy(void *handle) {
  imodel::destroy(static_cast<Handle *>(handle));
  return IMODEL_SWM_OK;
}

const char *imodel_swm_last_error(void *handle) {
  Handle *H = static_cast<Handle *>(handle);
  if (!H) return "NULL handle";
  return H->err.c_str();
}

}  // extern "C"

// ---- the moist shallow-water model ---------------------------------------------
namespace {
struct Moist {
  Handle *H = nullptr;  // the shallow-water handle: geometry, h and u
  int testcase = 0;
  int upw1 = 0;  // tracer advection "upw1" instead of "trsk"
  bool fp32 = false;  // FP32 handle: the f_ buffers instead of the FP64 ones
  double q0 = 0.0;
  double *th = nullptr, *ex20 = nullptr, *qv = nullptr, *qc = nullptr, *qr = nullptr;
  double *q[5][4] = {};  // per tracer: y_n, two stage buffers, RK accumulator
  double *uphi = nullptr;
  float *f_th = nullptr, *f_ex20 = nullptr, *f_qv = nullptr, *f_qc = nullptr, *f_qr = nullptr;
  float *f_q[5][4] = {};
  bool state_set = false;
  // one step's launches, captured once per dt and replayed
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0.0;
};

// host array (reference order, nv or ne values) -> device array (device order)
int moist_in(Handle *H, const double *src, double *dst, bool edges) {
  const int n = edges ? H->ne : H->nv;
  double *stage = edges ? H->d_stage_u : H->d_stage_h;
  CK(cudaMemcpyAsync(stage, src, sizeof(double) * n, cudaMemcpyHostToDevice, H->stream));
  imodel::launch_gather_in(n, edges ? H->d_edge_n2o : H->d_cell_n2o, stage, dst, 0.0, H->stream);
  CK(cudaGetLastError());
  return IMODEL_SWM_OK;
}
int moist_out(Handle *H, const double *src, double *dst, bool edges) {
  const int n = edges ? H->ne : H->nv;
  double *stage = edges ? H->d_stage_u : H->d_stage_h;
  imodel::launch_scatter_out(n, edges ? H->d_edge_n2o : H->d_cell_n2o, src, stage, 0.0,
                             H->d_flags, H->stream);
  CK(cudaMemcpyAsync(dst, stage, sizeof(double) * n, cudaMemcpyDeviceToHost, H->stream));
  CK(cudaGetLastError());
  return IMODEL_SWM_OK;
}
// the same into and out of FP32 device arrays, dst = src - shift and back
int moist_in32(Handle *H, const double *src, float *dst, bool edges, double shift) {
  const int n = edges ? H->ne : H->nv;
  double *stage = edges ? H->d_stage_u : H->d_stage_h;
  CK(cudaMemcpyAsync(stage, src, sizeof(double) * n, cudaMemcpyHostToDevice, H->stream));
  imodel::launch_gather_in32(n, edges ? H->d_edge_n2o : H->d_cell_n2o, stage, dst, shift,
                             H->stream);
  CK(cudaGetLastError());
  return IMODEL_SWM_OK;
}
int moist_out32(Handle *H, const float *src, double *dst, bool edges, double shift) {
  const int n = edges ? H->ne : H->nv;
  double *stage = edges ? H->d_stage_u : H->d_stage_h;
  imodel::launch_scatter_out32(n, edges ? H->d_edge_n2o : H->d_cell_n2o, src, stage, shift,
                               H->d_flags, H->stream);
  CK(cudaMemcpyAsync(dst, stage, sizeof(double) * n, cudaMemcpyDeviceToHost, H->stream));
  CK(cudaGetLastError());
  return IMODEL_SWM_OK;
}

// stage st of the RK4 loop reads y_n, a, b, a and writes a, b, a, y_n
template <class T>
T *stage_in(int st, T *yn, T *a, T *b) {
  return st == 0 ? yn : (st == 2 ? b : a);
}
template <class T>
T *stage_out(int st, T *yn, T *a, T *b) {
  return st == 0 ? a : (st == 1 ? b : (st == 2 ? a : yn));
}

// one step of an FP32 handle: the FP32 step's tendency (its tuned variant,
// tendencies only), then the moist kernels in FP32
void moist_step32(Moist *X, double dt) {
  Handle *H = X->H;
  imodel::Work<float> &W = H->W32;
  const float fdt = static_cast<float>(dt);
  const bool swm = X->testcase > 1;
  const int active = swm ? (0xF | (X->testcase == 2 ? 0x10 : 0)) : 0x10;
  {
    for (int st = 0; st < 4; ++st) {
      imodel::MoistArgs32 A;
      A.stage = st;
      A.dt = fdt;
      A.swm = swm ? 1 : 0;
      A.active = active;
      A.upw1 = X->upw1;
      A.h_ref = W.h_ref;
      const float *h_in = swm ? stage_in(st, W.yn_h, W.ya_h, W.yb_h) : W.yn_h;
      const float *u_in = swm ? stage_in(st, W.yn_u, W.ya_u, W.yb_u) : W.yn_u;
      if (swm) imodel::launch_stage32(H->M, W, h_in, u_in, nullptr, nullptr, -1, fdt, H->stream);
      A.h_in = h_in;
      A.u_in = u_in;
      A.tend_h = W.tend_h;
      A.tend_u = W.tend_u;
      A.yn_h = W.yn_h;
      A.acc_h = W.acc_h;
      A.h_out = stage_out(st, W.yn_h, W.ya_h, W.yb_h);
      A.yn_u = W.yn_u;
      A.acc_u = W.acc_u;
      A.u_out = stage_out(st, W.yn_u, W.ya_u, W.yb_u);
      for (int k = 0; k < 5; ++k) {
        float **q = X->f_q[k];
        const bool adv = (active >> k) & 1;
        A.q_in[k] = adv ? stage_in(st, q[0], q[1], q[2]) : q[0];
        A.q_yn[k] = q[0];
        A.q_acc[k] = q[3];
        A.q_out[k] = stage_out(st, q[0], q[1], q[2]);
      }
      A.th = X->f_th;
      A.ex20 = X->f_ex20;
      A.qv = X->f_qv;
      A.qc = X->f_qc;
      A.qr = X->f_qr;
      A.q0 = static_cast<float>(X->q0);
      A.flags = H->d_flags;
      imodel::launch_moist_stage32(H->M, A, H->stream);
    }
    imodel::launch_moist_q32(H->nv, W.yn_h, W.h_ref, X->f_q[1][0], X->f_q[2][0], X->f_q[3][0],
                             X->f_qv, X->f_qc, X->f_qr, H->d_flags, H->stream);
  }
}

// one step of an FP64 handle: the FP64 tendency (tendencies only), then
// the moist kernels
void moist_step64(Moist *X, double dt) {
  Handle *H = X->H;
  imodel::Work<double> &W = H->W64;
  const bool swm = X->testcase > 1;
  const int active = swm ? (0xF | (X->testcase == 2 ? 0x10 : 0)) : 0x10;
  // stage st reads y_n, a, b, a and writes a, b, a, y_n
  auto in = [](int st, double *yn, double *a, double *b) { return st == 0 ? yn : (st == 2 ? b : a); };
  auto out = [](int st, double *yn, double *a, double *b) {
    return st == 0 ? a : (st == 1 ? b : (st == 2 ? a : yn));
  };
  {
    for (int st = 0; st < 4; ++st) {
      imodel::MoistArgs A;
      A.stage = st;
      A.dt = dt;
      A.swm = swm ? 1 : 0;
      A.active = active;
      A.upw1 = X->upw1;
      const double *h_in = swm ? in(st, W.yn_h, W.ya_h, W.yb_h) : W.yn_h;
      const double *u_in = swm ? in(st, W.yn_u, W.ya_u, W.yb_u) : W.yn_u;
      if (swm)
        imodel::launch_stage64(H->M, W, h_in, u_in, nullptr, nullptr, -1, dt, H->stream);
      A.h_in = h_in;
      A.u_in = u_in;
      A.tend_h = W.tend_h;
      A.tend_u = W.tend_u;
      A.h_ed = W.h_ed;
      A.yn_h = W.yn_h;
      A.acc_h = W.acc_h;
      A.h_out = out(st, W.yn_h, W.ya_h, W.yb_h);
      A.yn_u = W.yn_u;
      A.acc_u = W.acc_u;
      A.u_out = out(st, W.yn_u, W.ya_u, W.yb_u);
      for (int k = 0; k < 5; ++k) {
        double **q = X->q[k];
        const bool adv = (active >> k) & 1;
        A.q_in[k] = adv ? in(st, q[0], q[1], q[2]) : q[0];
        A.q_yn[k] = q[0];
        A.q_acc[k] = q[3];
        A.q_out[k] = out(st, q[0], q[1], q[2]);
      }
      A.uphi = X->uphi;
      A.th = X->th;
      A.ex20 = X->ex20;
      A.qv = X->qv;
      A.qc = X->qc;
      A.qr = X->qr;
      A.q0 = X->q0;
      A.flags = H->d_flags;
      imodel::launch_moist_stage(H->M, A, H->stream);
    }
    imodel::launch_moist_q(H->nv, W.yn_h, X->q[1][0], X->q[2][0], X->q[3][0], X->qv, X->qc,
                           X->qr, H->d_flags, H->stream);
  }
}

// X->graph: one step's launches for this dt (captured anew when dt changes)
int moist_graph(Moist *X, double dt) {
  Handle *H = X->H;
  if (X->graph && X->graph_dt == dt) return IMODEL_SWM_OK;
  if (X->graph) {
    cudaGraphExecDestroy(X->graph);
    X->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
  if (X->fp32)
    moist_step32(X, dt);
  else
    moist_step64(X, dt);
  CK(cudaStreamEndCapture(H->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&X->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    X->graph = nullptr;
    return imodel::set_error(H, IMODEL_SWM_ECUDA,
                             std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  X->graph_dt = dt;
  return IMODEL_SWM_OK;
}
}  // namespace

extern "C" {

int imodel_moist_create(const imodel_swm_mesh *m, const imodel_moist_opts *o, void **handle) {
  if (!handle) return IMODEL_SWM_EINVAL;
  *handle = nullptr;
  Moist *X = new (std::nothrow) Moist();
  if (!X) return IMODEL_SWM_ENOMEM;
  X->H = new (std::nothrow) Handle();
  *handle = X;
  if (!X->H) return IMODEL_SWM_ENOMEM;
  Handle *H = X->H;
  if (!m || !o || !o->theta) return imodel::set_error(H, IMODEL_SWM_EINVAL, "mesh, opts and theta are required");
  if (o->testcase < 1 || o->testcase > 5)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "moist test cases are 1..5");
  if (o->advection != 0 && o->advection != 1)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "advection is 0 (trsk) or 1 (upw1)");
  if (o->precision != IMODEL_SWM_FP64 && o->precision != IMODEL_SWM_FP32)
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "precision is IMODEL_SWM_FP64 or IMODEL_SWM_FP32");
  imodel_swm_opts so{};
  so.precision = o->precision;
  so.testcase = o->testcase;
  so.bt = o->bt;
  so.device = o->device;
  int rc;
  try {
    rc = imodel::create(H, m, &so);
  } catch (const std::bad_alloc &) {
    rc = imodel::set_error(H, IMODEL_SWM_ENOMEM, "host allocation failed");
  }
  if (rc) return rc;
  X->testcase = o->testcase;
  X->upw1 = o->advection;
  X->q0 = o->q0;
  X->fp32 = o->precision == IMODEL_SWM_FP32;
  const size_t nv = H->nv, ne = H->ne;
  // theta and exp(20 theta) of qsat (moist_swm.f90:618-622): theta is fixed
  // in the RK4 path, so the exponential is formed once, here
  std::vector<double> ex(nv);
  for (size_t i = 0; i < nv; ++i) ex[i] = std::exp(20.0 * o->theta[i]);
  if (X->fp32) {
    for (float **p : {&X->f_th, &X->f_ex20, &X->f_qv, &X->f_qc, &X->f_qr})
      if ((rc = imodel::dalloc(H, p, nv))) return rc;
    for (int k = 0; k < 5; ++k)
      for (int b = 0; b < 4; ++b)
        if ((rc = imodel::dalloc(H, &X->f_q[k][b], nv))) return rc;
    if ((rc = moist_in32(H, o->theta, X->f_th, false, 0.0)) ||
        (rc = moist_in32(H, ex.data(), X->f_ex20, false, 0.0)))
      return rc;
  } else {
    for (double **p : {&X->th, &X->ex20, &X->qv, &X->qc, &X->qr})
      if ((rc = imodel::dalloc(H, p, nv))) return rc;
    for (int k = 0; k < 5; ++k)
      for (int b = 0; b < 4; ++b)
        if ((rc = imodel::dalloc(H, &X->q[k][b], nv))) return rc;
    if ((rc = imodel::dalloc(H, &X->uphi, 5 * ne))) return rc;
    if ((rc = moist_in(H, o->theta, X->th, false)) || (rc = moist_in(H, ex.data(), X->ex20, false)))
      return rc;
  }
  if (cudaStreamSynchronize(H->stream) != cudaSuccess)
    return imodel::set_error(H, IMODEL_SWM_ECUDA, "stream synchronize failed");
  return IMODEL_SWM_OK;
}

int imodel_moist_set_state(void *handle, const double *const y[7], const double *qv,
                           const double *qc, const double *qr) {
  Moist *X = static_cast<Moist *>(handle);
  if (!X || !X->H || !y || !qv || !qc || !qr) return IMODEL_SWM_EINVAL;
  Handle *H = X->H;
  if (H->nv == 0) return imodel::set_error(H, IMODEL_SWM_ESTATE, "handle was not created");
  for (int k = 0; k < 7; ++k)
    if (!y[k]) return IMODEL_SWM_EINVAL;
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc;
  if (X->fp32) {
    // h is stored as h - h_ref, h_ref the area-weighted mean of the first
    // state set (in FP32), as for the FP32 shallow-water handle
    if (!H->href_fixed) {
      double s = 0.0, a = 0.0;
      for (int i = 0; i < H->nv; ++i) {
        a += H->h_areag[i];
        s += H->h_areag[i] * y[0][i];
      }
      H->W32.h_ref = static_cast<float>(s / a);
      H->h_ref = static_cast<double>(H->W32.h_ref);
      H->href_fixed = true;
    }
    if ((rc = moist_in32(H, y[0], H->W32.yn_h, false, H->h_ref)) ||
        (rc = moist_in32(H, y[1], H->W32.yn_u, true, 0.0)))
      return rc;
    for (int k = 0; k < 5; ++k)
      if ((rc = moist_in32(H, y[2 + k], X->f_q[k][0], false, 0.0))) return rc;
    if ((rc = moist_in32(H, qv, X->f_qv, false, 0.0)) ||
        (rc = moist_in32(H, qc, X->f_qc, false, 0.0)) ||
        (rc = moist_in32(H, qr, X->f_qr, false, 0.0)))
      return rc;
  } else {
    if ((rc = moist_in(H, y[0], H->W64.yn_h, false)) || (rc = moist_in(H, y[1], H->W64.yn_u, true)))
      return rc;
    for (int k = 0; k < 5; ++k)
      if ((rc = moist_in(H, y[2 + k], X->q[k][0], false))) return rc;
    if ((rc = moist_in(H, qv, X->qv, false)) || (rc = moist_in(H, qc, X->qc, false)) ||
        (rc = moist_in(H, qr, X->qr, false)))
      return rc;
  }
  if (cudaStreamSynchronize(H->stream) != cudaSuccess)
    return imodel::set_error(H, IMODEL_SWM_ECUDA, "stream synchronize failed");
  X->state_set = true;
  return IMODEL_SWM_OK;
}

int imodel_moist_advance(void *handle, double dt, int32_t nsteps) {
  Moist *X = static_cast<Moist *>(handle);
  if (!X || !X->H) return IMODEL_SWM_EINVAL;
  Handle *H = X->H;
  if (!X->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  if (nsteps < 0 || !(dt > 0) || !std::isfinite(dt))
    return imodel::set_error(H, IMODEL_SWM_EINVAL, "bad dt or nsteps");
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc = moist_graph(X, dt);
  if (rc) return rc;
  for (int step = 0; step < nsteps; ++step)
    if (cudaGraphLaunch(X->graph, H->stream) != cudaSuccess)
      return imodel::set_error(H, IMODEL_SWM_ECUDA, "cudaGraphLaunch failed");
  if (cudaGetLastError() != cudaSuccess) return imodel::set_error(H, IMODEL_SWM_ECUDA, "launch failed");
  return imodel::check_flags(H);
}

int imodel_moist_get_state(void *handle, double *const y[7]) {
  Moist *X = static_cast<Moist *>(handle);
  if (!X || !X->H || !y) return IMODEL_SWM_EINVAL;
  Handle *H = X->H;
  if (!X->state_set) return imodel::set_error(H, IMODEL_SWM_ESTATE, "no state set");
  for (int k = 0; k < 7; ++k)
    if (!y[k]) return IMODEL_SWM_EINVAL;
  if (cudaSetDevice(H->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc;
  if (X->fp32) {
    if ((rc = moist_out32(H, H->W32.yn_h, y[0], false, H->h_ref)) ||
        (rc = moist_out32(H, H->W32.yn_u, y[1], true, 0.0)))
      return rc;
    for (int k = 0; k < 5; ++k)
      if ((rc = moist_out32(H, X->f_q[k][0], y[2 + k], false, 0.0))) return rc;
    return imodel::check_flags(H);
  }
  if ((rc = moist_out(H, H->W64.yn_h, y[0], false)) || (rc = moist_out(H, H->W64.yn_u, y[1], true)))
    return rc;
  for (int k = 0; k < 5; ++k)
    if ((rc = moist_out(H, X->q[k][0], y[2 + k], false))) return rc;
  return imodel::check_flags(H);
}

int imodel_moist_destroy(void *handle) {
  Moist *X = static_cast<Moist *>(handle);
  if (!X) return IMODEL_SWM_OK;
  if (X->graph) cudaGraphExecDestroy(X->graph);
  imodel::destroy(X->H);
  delete X;
  return IMODEL_SWM_OK;
}

const char *imodel_moist_last_error(void *handle) {
  Moist *X = static_cast<Moist *>(handle);
  return X && X->H ? X->H->err.c_str() : "null handle";
}

}  // extern "C"
