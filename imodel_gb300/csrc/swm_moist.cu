// FP64 kernels of the moist shallow-water model (moist_swm.f90) beside the
// shallow-water tendency of swm_k64.cu: the flux-form tracer advection of
// advmtd = "trsk", the thermal momentum source, the condensation sources and
// the RK4 stages of all seven fields.
//
// Compiled with --fmad=false and in the reference's operation order, so that
// the GPU equals the CPU oracle bit for bit.  The one transcendental of the
// sources, exp(20 theta) in qsat, is formed once on the host (theta keeps its
// initial value in the reference's RK4 path) and read here.
#include "swm_common.cuh"

namespace imodel {
namespace {

// constants.f90:45 -- eps = epsilon(1.) (float epsilon)
constexpr double kEps = 1.1920928955078125e-07;
// initialize_moist_swm_fields (moist_swm.f90:730-732)
constexpr double kLscale = 10.0, kGammaR = 0.001, kQprecip = 0.0001;

__device__ __forceinline__ double rk_stage(int stage, double k, double yn, double *acc, double dt) {
  // ode_rk4_moist_swm, moist_swm.f90:1880-1960
  if (stage == 0) {
    *acc = k;
    return yn + dt * k / 2.0;
  } else if (stage == 1) {
    *acc = *acc + 2.0 * k;
    return yn + dt * k / 2.0;
  } else if (stage == 2) {
    *acc = *acc + 2.0 * k;
    return yn + dt * k;
  }
  return yn + dt * (*acc + k) / 6.0;
}
// Fortran max(0, x) / min(a, b) as std::max / std::min evaluate them
__device__ __forceinline__ double fmax0(double x) { return (0.0 < x) ? x : 0.0; }
__device__ __forceinline__ double fminq(double a, double b) { return (b < a) ? b : a; }

// Edges: u q_e for every advanced tracer with advmtd = "trsk" (scalar_hx2ed
// + scalar_elem_product, divhx; "upw1" forms its fluxes in the cell
// kernel); with the shallow-water terms on, the thermal momentum source
// (source, moist_swm.f90:1299-1315) added to the momentum tendency and u's
// RK stage.
__global__ void __launch_bounds__(256) k_moist_edge(DevMesh M, MoistArgs A) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const int v1 = M.e_v[e], v2 = M.e_v[ne + e];
  const double ue = A.u_in[e];
  if (!A.upw1) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      if (!((A.active >> k) & 1)) continue;
      const double qe = (A.q_in[k][v1] + A.q_in[k][v2]) * 0.5;
      A.uphi[static_cast<size_t>(k) * ne + e] = ue * qe;
    }
  }
  if (!A.swm) return;
  const double l = M.e_leng[e], erad = M.erad, grav = M.grav;
  double g = A.h_in[v2] * A.q_in[0][v2] - A.h_in[v1] * A.q_in[0][v1];
  g = g / l / erad;
  const double hed = A.h_ed[e];
  double gpi_oh = 0.0;
  if (fabs(hed) < kEps / 100000.0)
    atomicOr(A.flags, 1);
  else
    gpi_oh = g / hed;
  double gb = M.c_bt[v2] - M.c_bt[v1];
  gb = gb / l / erad;
  const double th_ed = (A.th[v1] + A.th[v2]) * 0.5;
  const double su = (grav * 0.5) * gpi_oh + grav * (th_ed * gb);
  const double momeq = A.tend_u[e] + su;
  A.u_out[e] = rk_stage(A.stage, momeq, A.yn_u[e], A.acc_u + e, A.dt);
}

// Cells: the divergence of each advected tracer's flux (div_hx, or
// div_hx_upw1 with the upwind fluxes formed here), the
// condensation, evaporation and precipitation sources (source, :1317-1351)
// and the RK stages of h and the tracers.
__global__ void __launch_bounds__(256) k_moist_cell(DevMesh M, MoistArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv, ne = M.ne;
  if (i >= nv) return;
  double hs[4] = {0.0, 0.0, 0.0, 0.0};
  if (A.swm) {
    A.h_out[i] = rk_stage(A.stage, A.tend_h[i], A.yn_h[i], A.acc_h + i, A.dt);
    const double hi = A.h_in[i];
    const double qs = A.q0 * A.ex20[i] / ((hi + M.c_bt[i]) * M.grav);
    double gamma_v = 1.0 + kLscale * (20.0 * qs);
    gamma_v = 1.0 / gamma_v;
    const double qv = A.qv[i], qc = A.qc[i];
    double dqv = gamma_v * (qv - qs);
    dqv = fmax0(dqv) / A.dt;
    double dqc = fmax0(-gamma_v * (qv - qs));
    dqc = fminq(qc, dqc) / A.dt;
    const double dqr = fmax0(kGammaR * (qc - kQprecip)) / A.dt;
    hs[1] = hi * (dqc - dqv);
    hs[2] = hi * (dqv - dqc - dqr);
    hs[3] = hi * dqr;
    hs[0] = hi * (kLscale * (dqv - dqc));
  }
  const int n = M.c_nnb[i];
  const double A_i = M.c_areag[i], erad = M.erad;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    if (!((A.active >> k) & 1)) continue;
    double d = 0.0;
    if (A.upw1) {
      // div_hx_upw1: c_sd = ttgout l_e, so (u c_sd) q is the reference's
      // ((ttgout u) l_e) q bit for bit; the cell's own value where the
      // flux leaves it (ttgout u > 0), the neighbour's where it enters
      for (int j = 0; j < n; ++j) {
        const int e = M.c_ed[j * nv + i];
        const double sd = M.c_sd[j * nv + i], ue = A.u_in[e];
        const double out = sd > 0.0 ? ue : -ue;
        // the neighbour across slot j: the other end of edge e (mesh%v(i)%nb(j))
        const int a = M.e_v[e], b = M.e_v[ne + e];
        const double qu = out > 0.0 ? A.q_in[k][i] : A.q_in[k][a == i ? b : a];
        d = d + ue * sd * qu;
      }
    } else {
      const double *uphi = A.uphi + static_cast<size_t>(k) * ne;
      for (int j = 0; j < n; ++j) d = d + uphi[M.c_ed[j * nv + i]] * M.c_sd[j * nv + i];
    }
    double t = -(d / A_i / erad);
    if (A.swm && k < 4) t = t + hs[k];
    A.q_out[k][i] = rk_stage(A.stage, t, A.q_yn[k][i], A.q_acc[k] + i, A.dt);
  }
}

// after a step: qv, qc, qr = h qv / h etc. (scalar_elem_divide, with its
// guard), the fields the next step's sources read
__global__ void k_moist_q(int nv, const double *__restrict__ h, const double *__restrict__ hqv,
                          const double *__restrict__ hqc, const double *__restrict__ hqr,
                          double *__restrict__ qv, double *__restrict__ qc,
                          double *__restrict__ qr, int *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const double hi = h[i];
  if (fabs(hi) < kEps / 100000.0) {
    atomicOr(flags, 1);
    return;
  }
  qv[i] = hqv[i] / hi;
  qc[i] = hqc[i] / hi;
  qr[i] = hqr[i] / hi;
}

// ---- FP32 --------------------------------------------------------------------
// The same model beside the FP32 step (any of its variants, tendencies
// only): h is stored as h - h_ref, so h itself is h_ref + h_d where the
// sources and the thermal term need it; the gradient of h (h theta) is
// formed as
//   h2 Q2 - h1 Q1 = (h_d2 - h_d1) (Q1 + Q2) / 2 + (Q2 - Q1) (h1 + h2) / 2
// (exact in real arithmetic), which keeps the difference of the depths free
// of h_ref's rounding.  The divergences use the cells' folded coefficients
// c_div32 = ttgout l_e / (A erad), the gradients e_grad32 = 1 / (l erad).
// Each cell forms the tracer flux of its edges itself from its neighbour
// across the edge (c_nb): u_e (q_i + q_nb) / 2 with "trsk", the upwind
// value with "upw1"; the two cells of an edge form the same flux, since
// q_i + q_nb and q_nb + q_i round alike, so no flux array goes through
// memory.

__device__ __forceinline__ float rk_stage32m(int stage, float k, float yn, float *acc, float dt) {
  if (stage == 0) {
    *acc = k;
    return yn + dt * k * 0.5f;
  } else if (stage == 1) {
    *acc = *acc + 2.0f * k;
    return yn + dt * k * 0.5f;
  } else if (stage == 2) {
    *acc = *acc + 2.0f * k;
    return yn + dt * k;
  }
  return yn + dt * (*acc + k) * (1.0f / 6.0f);
}

// the thermal momentum source and u's RK stage (shallow-water cases only)
__global__ void __launch_bounds__(256) k_moist_edge32(DevMesh M, MoistArgs32 A) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const int v1 = __ldg(&M.e_v[e]), v2 = __ldg(&M.e_v[ne + e]);
  const float gr = __ldg(&M.e_grad32[e]), grav = static_cast<float>(M.grav);
  const float hd1 = A.h_in[v1], hd2 = A.h_in[v2];
  const float Q1 = A.q_in[0][v1], Q2 = A.q_in[0][v2];
  const float h1 = A.h_ref + hd1, h2 = A.h_ref + hd2;
  const float g = ((hd2 - hd1) * (Q1 + Q2) * 0.5f + (Q2 - Q1) * (h1 + h2) * 0.5f) * gr;
  // scalar_hx2ed of h
  const float hed = A.h_ref + 0.5f * (hd1 + hd2);
  float gpi_oh = 0.0f;
  if (fabsf(hed) < 1.1920928955078125e-12f)
    atomicOr(A.flags, 1);
  else
    gpi_oh = g / hed;
  const float gb = (__ldg(&M.c_bt32[v2]) - __ldg(&M.c_bt32[v1])) * gr;
  const float th_ed = (A.th[v1] + A.th[v2]) * 0.5f;
  const float su = (grav * 0.5f) * gpi_oh + grav * (th_ed * gb);
  const float momeq = A.tend_u[e] + su;
  A.u_out[e] = rk_stage32m(A.stage, momeq, A.yn_u[e], A.acc_u + e, A.dt);
}

__global__ void __launch_bounds__(256) k_moist_cell32(DevMesh M, MoistArgs32 A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  float hs[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (A.swm) {
    A.h_out[i] = rk_stage32m(A.stage, A.tend_h[i], A.yn_h[i], A.acc_h + i, A.dt);
    const float hi = A.h_ref + A.h_in[i];
    const float qs = A.q0 * A.ex20[i] / ((hi + __ldg(&M.c_bt32[i])) * static_cast<float>(M.grav));
    const float gamma_v = 1.0f / (1.0f + kLscale * (20.0f * qs));
    const float qv = A.qv[i], qc = A.qc[i];
    const float r = gamma_v * (qv - qs);
    const float dqv = fmaxf(r, 0.0f) / A.dt;
    const float dqc = fminf(qc, fmaxf(-r, 0.0f)) / A.dt;
    const float dqr = fmaxf(static_cast<float>(kGammaR) * (qc - static_cast<float>(kQprecip)), 0.0f) / A.dt;
    hs[1] = hi * (dqc - dqv);
    hs[2] = hi * (dqv - dqc - dqr);
    hs[3] = hi * dqr;
    hs[0] = hi * (static_cast<float>(kLscale) * (dqv - dqc));
  }
  // the cell's edges: the normal velocity times c_div32, and the neighbour
  const int n = M.c_nnb[i];
  float w[6];
  int nb[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    w[j] = 0.0f;
    nb[j] = i;
    if (j < n) {
      w[j] = A.u_in[__ldg(&M.c_ed[j * nv + i])] * __ldg(&M.c_div32[j * nv + i]);
      nb[j] = __ldg(&M.c_nb[j * nv + i]);
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    if (!((A.active >> k) & 1)) continue;
    const float *q = A.q_in[k];
    const float qi = q[i];
    float d = 0.0f;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j >= n) continue;
      const float qn = q[nb[j]];
      // "upw1": the cell's own value where the flux leaves it (w > 0)
      const float qf = A.upw1 ? (w[j] > 0.0f ? qi : qn) : (qi + qn) * 0.5f;
      d += w[j] * qf;
    }
    float t = -d;
    if (A.swm && k < 4) t = t + hs[k];
    A.q_out[k][i] = rk_stage32m(A.stage, t, A.q_yn[k][i], A.q_acc[k] + i, A.dt);
  }
}

__global__ void k_moist_q32(int nv, const float *__restrict__ hd, float h_ref,
                            const float *__restrict__ hqv, const float *__restrict__ hqc,
                            const float *__restrict__ hqr, float *__restrict__ qv,
                            float *__restrict__ qc, float *__restrict__ qr, int *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float hi = h_ref + hd[i];
  if (fabsf(hi) < 1.1920928955078125e-12f) {
    atomicOr(flags, 1);
    return;
  }
  qv[i] = hqv[i] / hi;
  qc[i] = hqc[i] / hi;
  qr[i] = hqr[i] / hi;
}

inline int nblocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void launch_moist_stage32(const DevMesh &M, const MoistArgs32 &A, cudaStream_t s) {
  if (A.swm) k_moist_edge32<<<nblocks(M.ne, 256), 256, 0, s>>>(M, A);
  k_moist_cell32<<<nblocks(M.nv, 256), 256, 0, s>>>(M, A);
}

void launch_moist_q32(int nv, const float *hd, float h_ref, const float *hqv, const float *hqc,
                      const float *hqr, float *qv, float *qc, float *qr, int *flags,
                      cudaStream_t s) {
  k_moist_q32<<<nblocks(nv, 256), 256, 0, s>>>(nv, hd, h_ref, hqv, hqc, hqr, qv, qc, qr, flags);
}

void launch_moist_stage(const DevMesh &M, const MoistArgs &A, cudaStream_t s) {
  k_moist_edge<<<nblocks(M.ne, 256), 256, 0, s>>>(M, A);
  k_moist_cell<<<nblocks(M.nv, 256), 256, 0, s>>>(M, A);
}

void launch_moist_q(int nv, const double *h, const double *hqv, const double *hqc,
                    const double *hqr, double *qv, double *qc, double *qr, int *flags,
                    cudaStream_t s) {
  k_moist_q<<<nblocks(nv, 256), 256, 0, s>>>(nv, h, hqv, hqc, hqr, qv, qc, qr, flags);
}

}  // namespace imodel
