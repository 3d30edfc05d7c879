// FP64 kernels in the reference's operation order, plus the layout
// permutations and the compensated FP64 integrals.
//
// This translation unit is compiled with --fmad=false: every product and sum
// below is rounded on its own, as in the Fortran built without contraction,
// so that the FP64 step reproduces the reference arithmetic of
// src/swm.f90:2416-2683 and src/swm_operators.f90 bit for bit.
#include "imodel_swm.h"
#include "swm_common.cuh"

namespace imodel {
namespace {

// constants.f90:45 -- eps = epsilon(1.) (float epsilon)
constexpr double kEps = 1.1920928955078125e-07;

template <class T>
__device__ __forceinline__ T rk_stage(int stage, T k, T yn, T *acc, T dt) {
  // ode_rk4, swm.f90:2647-2678
  if (stage == 0) {
    *acc = k;
    return yn + dt * k / T(2);
  } else if (stage == 1) {
    *acc = *acc + T(2) * k;
    return yn + dt * k / T(2);
  } else if (stage == 2) {
    *acc = *acc + T(2) * k;
    return yn + dt * k;
  }
  return yn + dt * (*acc + k) / T(6);
}

// vort_tr (:551-611) + scalar_hx2tr (:229-284) + scalar_elem_divide (:1579);
// the depth at the triangle by the scheme's interpolation (swm.f90:2459-2464):
// kite areas (trsk), barycentric weights of the circumcentre (bary, pxt16) or
// scalar_edtr2trcc of h_ed (:286-343, gass18, which also keeps eta and h_tr
// for the rhombus PV)
__global__ void __launch_bounds__(256) k_tri64(DevMesh M, const double *__restrict__ h,
                                               const double *__restrict__ u,
                                               double *__restrict__ q_tr, int pv_on,
                                               int *flags, const double *__restrict__ kt,
                                               double *__restrict__ coefvort, int scheme,
                                               double *__restrict__ eta_t,
                                               double *__restrict__ h_trs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.nt;
  if (t >= nt) return;
  double e = 0.0;
#pragma unroll
  for (int s = 0; s < 3; ++s) e = e + u[M.t_ed[s * nt + t]] * M.t_lt[s * nt + t];
  const double A = M.t_areag[t];
  e = e / A / M.erad;
  // with diffusion on: rel_vort_tr(u) (:780-827) is this sum before f is
  // added; diffusion_ed's K_tr zeta
  if (coefvort) coefvort[t] = kt[t] * e;
  e = e + M.t_f[t];
  double ht = 0.0;
  if (scheme == IMODEL_SWM_PXT16) {
#pragma unroll
    for (int s = 0; s < 3; ++s) ht = ht + M.t_bary[s * nt + t] * h[M.t_v[s * nt + t]];
  } else if (scheme == IMODEL_SWM_GASS18) {
    const int ne = M.ne;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int ed = M.t_ed[s * nt + t];
      const double he = (h[M.e_v[ed]] + h[M.e_v[ne + ed]]) * 0.5;
      ht = ht + M.t_edarea[s * nt + t] * he;
    }
    ht = ht / A;
    eta_t[t] = e;
    h_trs[t] = ht;
  } else {
#pragma unroll
    for (int s = 0; s < 3; ++s) ht = ht + M.t_kite[s * nt + t] * h[M.t_v[s * nt + t]];
    ht = ht / A;
  }
  double q = 0.0;
  if (pv_on) {
    if (fabs(ht) < kEps / 100000.0)
      atomicOr(flags, 1);
    else
      q = e / ht;
  }
  q_tr[t] = q;
}

// proj_vec_sphere (smeshpack.f90:4419-4433): v - (v . p) p / |p|
__device__ __forceinline__ void proj_sphere(double &v0, double &v1, double &v2, double p0,
                                            double p1, double p2) {
  const double vp = v0 * p0 + v1 * p1 + v2 * p2;
  const double np = sqrt(p0 * p0 + p1 * p1 + p2 * p2);
  v0 = v0 - vp * p0 / np;
  v1 = v1 - vp * p1 / np;
  v2 = v2 - vp * p2 / np;
}

// grad_tr2ed(q_tr) (:1427-1463), the PV gradient across each edge
__global__ void __launch_bounds__(256) k_qgrad64(DevMesh M, const double *__restrict__ q_tr,
                                                 double *__restrict__ qge) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  double g = M.e_sgtg[e] * (q_tr[M.e_sh[ne + e]] - q_tr[M.e_sh[e]]);
  qge[e] = g / M.e_dleng[e] / M.erad;
}

// The two reconstructions apvm (:1465-1543) reads.  Blocks [0, nbt): the
// PV gradient at the triangles, vector_edtr2tr_perot (:408-452) of qge;
// dsign(1, tr%nr) = -tr%tg (smeshpack.f90:853-859), the sign of t_lt.
// The blocks after: the velocity at the cells, vector_edhx2hx_perot
// (:454-509, HTC, hx%areag); ttgout is the sign of c_sd.
__global__ void __launch_bounds__(256) k_apvm64(DevMesh M, const double *__restrict__ qge,
                                                const double *__restrict__ u,
                                                double *__restrict__ qg,
                                                double *__restrict__ vhx, int nbt) {
  const int ne = M.ne;
  if (static_cast<int>(blockIdx.x) < nbt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = M.nt;
    if (t >= nt) return;
    const double c0 = M.t_c[t], c1 = M.t_c[nt + t], c2 = M.t_c[2 * nt + t];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int ed = M.t_ed[s * nt + t];
      const double sg = (M.t_lt[s * nt + t] < 0.0 ? 1.0 : -1.0) * qge[ed];
      const double l = M.e_leng[ed];
      v0 = v0 + sg * (M.e_c[ed] - c0) * l;
      v1 = v1 + sg * (M.e_c[ne + ed] - c1) * l;
      v2 = v2 + sg * (M.e_c[2 * ne + ed] - c2) * l;
    }
    const double A = M.t_areag[t];
    v0 = v0 / A;
    v1 = v1 / A;
    v2 = v2 / A;
    proj_sphere(v0, v1, v2, c0, c1, c2);
    qg[t] = v0;
    qg[nt + t] = v1;
    qg[2 * nt + t] = v2;
  } else {
    const int i = (blockIdx.x - nbt) * blockDim.x + threadIdx.x;
    const int nv = M.nv;
    if (i >= nv) return;
    const double p0 = M.c_p[i], p1 = M.c_p[nv + i], p2 = M.c_p[2 * nv + i];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    const int n = M.c_nnb[i];
    for (int j = 0; j < n; ++j) {
      const int ed = M.c_ed[j * nv + i];
      const double su = (M.c_sd[j * nv + i] < 0.0 ? -1.0 : 1.0) * u[ed];
      const double d = M.e_dleng[ed];
      v0 = v0 + su * (M.e_c[ed] - p0) * d;
      v1 = v1 + su * (M.e_c[ne + ed] - p1) * d;
      v2 = v2 + su * (M.e_c[2 * ne + ed] - p2) * d;
    }
    const double A = M.c_areag[i];
    v0 = v0 / A;
    v1 = v1 / A;
    v2 = v2 / A;
    proj_sphere(v0, v1, v2, p0, p1, p2);
    vhx[i] = v0;
    vhx[nv + i] = v1;
    vhx[2 * nv + i] = v2;
  }
}

// scalar_hx2ed (:89-97), scalar_elem_product (:1546), scalar_tr2ed (:124-176:
// the plain average for trsk, circumcentre-distance weights for bary) or,
// for gass18, scalar_elem_divide of the rhombus averages of eta and h_tr
// (swm.f90:2475-2480); with qg != NULL the apvm correction of q_ed
// (:1495-1502), coef = pvspar dt
__global__ void __launch_bounds__(256) k_edge_pre64(DevMesh M, const double *__restrict__ h,
                                                    const double *__restrict__ u,
                                                    const double *__restrict__ q_tr,
                                                    double *__restrict__ h_ed,
                                                    double *__restrict__ uh,
                                                    double *__restrict__ q_ed,
                                                    const double *__restrict__ qg,
                                                    const double *__restrict__ vhx,
                                                    double coef, int scheme,
                                                    const double *__restrict__ eta_t,
                                                    const double *__restrict__ h_trs,
                                                    int pv_on, int *flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const double he = (h[M.e_v[e]] + h[M.e_v[ne + e]]) * 0.5;
  h_ed[e] = he;
  uh[e] = u[e] * he;
  const int t1 = M.e_sh[e], t2 = M.e_sh[ne + e];
  double q;
  if (scheme == IMODEL_SWM_PXT16) {
    const double d1 = M.e_dist[e], d2 = M.e_dist[ne + e];
    q = (d2 * q_tr[t1] + d1 * q_tr[t2]) / (d1 + d2);
  } else if (scheme == IMODEL_SWM_GASS18) {
    const double a1 = M.t_areag[t1], a2 = M.t_areag[t2];
    const double eta_ed = (a1 * eta_t[t1] + a2 * eta_t[t2]) / (a1 + a2);
    const double h_rhb = (a1 * h_trs[t1] + a2 * h_trs[t2]) / (a1 + a2);
    q = 0.0;
    if (pv_on) {
      if (fabs(h_rhb) < kEps / 100000.0)
        atomicOr(flags, 1);
      else
        q = eta_ed / h_rhb;
    }
  } else {
    q = 0.5 * (q_tr[t1] + q_tr[t2]);
  }
  if (qg) {
    const int nt = M.nt, nv = M.nv;
    const int c1 = M.e_v[e], c2 = M.e_v[ne + e];
    const double a0 = qg[t1] + qg[t2], a1 = qg[nt + t1] + qg[nt + t2],
                 a2 = qg[2 * nt + t1] + qg[2 * nt + t2];
    const double b0 = vhx[c1] + vhx[c2], b1 = vhx[nv + c1] + vhx[nv + c2],
                 b2 = vhx[2 * nv + c1] + vhx[2 * nv + c2];
    q = q - coef * (a0 * b0 + a1 * b1 + a2 * b2);
  }
  q_ed[e] = q;
}

// div_hx(uh) (:613-661), kinetic_energy_hx trsk (:1162-1171), Bernoulli
// potential (swm.f90:2533-2536) and the mass-equation RK stage
__global__ void __launch_bounds__(256) k_cell64(DevMesh M, const double *__restrict__ h,
                                                const double *__restrict__ u,
                                                const double *__restrict__ uh,
                                                double *__restrict__ bern,
                                                const double *__restrict__ yn,
                                                double *__restrict__ acc,
                                                double *__restrict__ yout,
                                                double *__restrict__ tend, int stage,
                                                double dt, const double *__restrict__ kcv,
                                                double *__restrict__ coefdiv, int perot_ke) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  const int n = M.c_nnb[i];
  double d = 0.0, k = 0.0, du = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = M.c_ed[j * nv + i];
    d = d + uh[e] * M.c_sd[j * nv + i];
    const double ue = u[e];
    k = k + M.e_kew[e] * (ue * ue);
    if (coefdiv) du = du + ue * M.c_sd[j * nv + i];
  }
  // with diffusion on: div_hx(u) (:613-661), diffusion_ed's K div u
  if (coefdiv) coefdiv[i] = kcv[i] * (du / M.c_areag[i] / M.erad);
  const double divuh = d / M.c_areag[i] / M.erad;
  double ke;
  if (perot_ke) {
    // kinetic_energy_hx, perhx branch (:1172-1173): half the squared
    // vector_edhx2hx_perot (:454-509, HTC) of u
    const int ne = M.ne;
    const double p0 = M.c_p[i], p1 = M.c_p[nv + i], p2 = M.c_p[2 * nv + i];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int j = 0; j < n; ++j) {
      const int ed = M.c_ed[j * nv + i];
      const double su = (M.c_sd[j * nv + i] < 0.0 ? -1.0 : 1.0) * u[ed];
      const double dl = M.e_dleng[ed];
      v0 = v0 + su * (M.e_c[ed] - p0) * dl;
      v1 = v1 + su * (M.e_c[ne + ed] - p1) * dl;
      v2 = v2 + su * (M.e_c[2 * ne + ed] - p2) * dl;
    }
    const double A = M.c_areag[i];
    v0 = v0 / A;
    v1 = v1 / A;
    v2 = v2 / A;
    proj_sphere(v0, v1, v2, p0, p1, p2);
    ke = (v0 * v0 + v1 * v1 + v2 * v2) / 2.0;
  } else {
    ke = k / M.c_cellarea[i];
  }
  bern[i] = M.grav * (h[i] + M.c_bt[i]) + ke;
  const double masseq = -divuh;
  if (stage < 0)
    tend[i] = masseq;
  else
    yout[i] = rk_stage(stage, masseq, yn[i], acc + i, dt);
}

// grad_ed (:511-548) + coriolis_ed TRSK (:1283-1308) and the momentum RK stage
__global__ void __launch_bounds__(256) k_edge64(DevMesh M, const double *__restrict__ bern,
                                                const double *__restrict__ uh,
                                                const double *__restrict__ q_ed,
                                                const double *__restrict__ yn,
                                                double *__restrict__ acc,
                                                double *__restrict__ yout,
                                                double *__restrict__ tend, int stage,
                                                double dt, int mom_on,
                                                const double *__restrict__ dif1,
                                                const double *__restrict__ dif2,
                                                const int32_t *__restrict__ stq) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const double l = M.e_leng[e];
  double g = bern[M.e_v[ne + e]] - bern[M.e_v[e]];
  g = g / l / M.erad;
  const double qe = q_ed[e];
  const int ns = M.e_nst[e];
  double q = 0.0;
  for (int s = 0; s < ns; ++s) {
    const int k = M.e_stk[s * ne + e];
    // gass18 (:1378-1410): the PV of the edge connecting e and k when there
    // is one (stq != NULL), else the TRSK average
    const int c3 = stq ? stq[s * ne + e] : -1;
    const double qtmp = c3 >= 0 ? q_ed[c3] : 0.5 * (qe + q_ed[k]);
    q = q + uh[k] * qtmp * M.e_dleng[k] * M.e_stw[s * ne + e];
  }
  q = q / l;
  double momeq = -g - q;
  // diffusion, then hyperdiffusion (swm.f90:2578-2589)
  if (dif1) momeq = momeq + dif1[e];
  if (dif2) momeq = momeq - dif2[e];
  if (!mom_on) momeq = 0.0;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage(stage, momeq, yn[e], acc + e, dt);
}

// dtred: vector_edhx2tr_perot (:345-406, HTC) of uh at the triangle
// circumcentres, cross(tr%c, v) / tr%areag, times q_tr (vector_elem_product,
// :1617-1649); signcor = dsign(1, tr%tg) is the sign of t_lt
__global__ void __launch_bounds__(256) k_vhq64(DevMesh M, const double *__restrict__ uh,
                                               const double *__restrict__ q_tr,
                                               double *__restrict__ vhq) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.nt, ne = M.ne;
  if (t >= nt) return;
  const double c0 = M.t_c[t], c1 = M.t_c[nt + t], c2 = M.t_c[2 * nt + t];
  double v0 = 0.0, v1 = 0.0, v2 = 0.0;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const int ed = M.t_ed[s * nt + t];
    const double su = (M.t_lt[s * nt + t] < 0.0 ? -1.0 : 1.0) * uh[ed];
    const double l = M.e_leng[ed];
    v0 = v0 + su * (M.e_c[ed] - c0) * l;
    v1 = v1 + su * (M.e_c[ne + ed] - c1) * l;
    v2 = v2 + su * (M.e_c[2 * ne + ed] - c2) * l;
  }
  const double w0 = c1 * v2 - c2 * v1, w1 = c2 * v0 - c0 * v2, w2 = c0 * v1 - c1 * v0;
  const double A = M.t_areag[t], q = q_tr[t];
  vhq[t] = w0 / A * q;
  vhq[nt + t] = w1 / A * q;
  vhq[2 * nt + t] = w2 / A * q;
}

// grad_ed (:511-548) + coriolis_ed's dtred (:1310-1329) or pered
// (:1330-1377) branch, HTC, and the momentum RK stage
__global__ void __launch_bounds__(256) k_edge64r(DevMesh M, const double *__restrict__ bern,
                                                 const double *__restrict__ uh,
                                                 const double *__restrict__ q_ed,
                                                 const double *__restrict__ vhq,
                                                 const double *__restrict__ yn,
                                                 double *__restrict__ acc,
                                                 double *__restrict__ yout,
                                                 double *__restrict__ tend, int stage,
                                                 double dt, int mom_on,
                                                 const double *__restrict__ dif1,
                                                 const double *__restrict__ dif2, int scheme) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne, nv = M.nv, nt = M.nt;
  if (e >= ne) return;
  const double l = M.e_leng[e];
  double g = bern[M.e_v[ne + e]] - bern[M.e_v[e]];
  g = g / l / M.erad;
  double v0, v1, v2;
  if (scheme == IMODEL_SWM_DTRED) {
    // the dual-triangle reconstructions of the edge's two triangles,
    // weighted by the other triangle's circumcentre distance
    const int k1 = M.e_sh[e], k2 = M.e_sh[ne + e];
    const double d1 = M.e_dist[e], d2 = M.e_dist[ne + e];
    v0 = (d2 * vhq[k1] + d1 * vhq[k2]) / (d1 + d2);
    v1 = (d2 * vhq[nt + k1] + d1 * vhq[nt + k2]) / (d1 + d2);
    v2 = (d2 * vhq[2 * nt + k1] + d1 * vhq[2 * nt + k2]) / (d1 + d2);
  } else {
    // pered: at each of the edge's cells the Perot reconstruction of
    // uh (q_e + q_k) / 2 over the cell's edges, projected on the tangent
    // plane; their average
    const double qe = q_ed[e];
    double vc[2][3];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int c = M.e_v[i * ne + e];
      const double p0 = M.c_p[c], p1 = M.c_p[nv + c], p2 = M.c_p[2 * nv + c];
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
      const int n = M.c_nnb[c];
      for (int j = 0; j < n; ++j) {
        const int l2 = M.c_ed[j * nv + c];
        const double qtmp = 0.5 * (qe + q_ed[l2]);
        const double f = (M.c_sd[j * nv + c] < 0.0 ? -1.0 : 1.0) * uh[l2] * qtmp;
        const double d = M.e_dleng[l2];
        a0 = a0 + f * (M.e_c[l2] - p0) * d;
        a1 = a1 + f * (M.e_c[ne + l2] - p1) * d;
        a2 = a2 + f * (M.e_c[2 * ne + l2] - p2) * d;
      }
      const double A = M.c_areag[c];
      a0 = a0 / A;
      a1 = a1 / A;
      a2 = a2 / A;
      proj_sphere(a0, a1, a2, p0, p1, p2);
      vc[i][0] = a0;
      vc[i][1] = a1;
      vc[i][2] = a2;
    }
    v0 = 0.5 * vc[0][0] + 0.5 * vc[1][0];
    v1 = 0.5 * vc[0][1] + 0.5 * vc[1][1];
    v2 = 0.5 * vc[0][2] + 0.5 * vc[1][2];
  }
  proj_sphere(v0, v1, v2, M.e_c[e], M.e_c[ne + e], M.e_c[2 * ne + e]);
  const double q = -(v0 * M.e_nr[e] + v1 * M.e_nr[ne + e] + v2 * M.e_nr[2 * ne + e]);
  double momeq = -g - q;
  if (dif1) momeq = momeq + dif1[e];
  if (dif2) momeq = momeq - dif2[e];
  if (!mom_on) momeq = 0.0;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage(stage, momeq, yn[e], acc + e, dt);
}

// diffusion_ed (swm_operators.f90:855-895), first half: coefdiv = K
// div_hx(x) at the cells (blocks [0, nbc)), coefvort = K_tr rel_vort_tr(x)
// at the triangles (the blocks after), HTC branches of div_hx (:613-661) and
// rel_vort_tr (:780-827)
__global__ void __launch_bounds__(256) k_difcv64(DevMesh M, const double *__restrict__ x,
                                                 const double *__restrict__ kcv,
                                                 const double *__restrict__ kt,
                                                 double *__restrict__ coefdiv,
                                                 double *__restrict__ coefvort, int nbc) {
  if (static_cast<int>(blockIdx.x) < nbc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nv = M.nv;
    if (i >= nv) return;
    const int n = M.c_nnb[i];
    double d = 0.0;
    for (int j = 0; j < n; ++j) d = d + x[M.c_ed[j * nv + i]] * M.c_sd[j * nv + i];
    const double divx = d / M.c_areag[i] / M.erad;
    coefdiv[i] = kcv[i] * divx;
  } else {
    const int t = (blockIdx.x - nbc) * blockDim.x + threadIdx.x;
    const int nt = M.nt;
    if (t >= nt) return;
    double z = 0.0;
#pragma unroll
    for (int s = 0; s < 3; ++s) z = z + x[M.t_ed[s * nt + t]] * M.t_lt[s * nt + t];
    z = z / M.t_areag[t] / M.erad;
    coefvort[t] = kt[t] * z;
  }
}

// second half: lap = grad_ed(coefdiv) - grad_ed_tg(coefvort) (grad_ed
// :511-548, grad_ed_tg :738-777, HTC)
__global__ void __launch_bounds__(256) k_diflap64(DevMesh M, const double *__restrict__ coefdiv,
                                                  const double *__restrict__ coefvort,
                                                  double *__restrict__ lap) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  double g = coefdiv[M.e_v[ne + e]] - coefdiv[M.e_v[e]];
  g = g / M.e_leng[e] / M.erad;
  double gt = M.e_sgtg[e] * (coefvort[M.e_sh[ne + e]] - coefvort[M.e_sh[e]]);
  gt = gt / (M.e_dleng[e] * M.erad);
  lap[e] = g - gt;
}

// the coefficients swm.f90:169-205 sets: at the cells the coefficient field
// kf (device order; NULL: the constant k), at the triangles its
// scalar_hx2tr (:258-263); both then sqrt for hyperdiffusion
__global__ void k_dif_coefs(DevMesh M, const double *__restrict__ kf, double k, int take_sqrt,
                            double *__restrict__ kc64, float *__restrict__ kc32,
                            double *__restrict__ kt64, float *__restrict__ kt32, int nbc) {
  if (static_cast<int>(blockIdx.x) < nbc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.nv) return;
    double f = kf ? kf[i] : k;
    if (take_sqrt) f = sqrt(f);
    kc64[i] = f;
    if (kc32) kc32[i] = static_cast<float>(f);
  } else {
    const int t = (blockIdx.x - nbc) * blockDim.x + threadIdx.x;
    const int nt = M.nt;
    if (t >= nt) return;
    double f = 0.0;
#pragma unroll
    for (int s = 0; s < 3; ++s) f = f + M.t_kite[s * nt + t] * (kf ? kf[M.t_v[s * nt + t]] : k);
    f = f / M.t_areag[t];
    if (take_sqrt) f = sqrt(f);
    kt64[t] = f;
    if (kt32) kt32[t] = static_cast<float>(f);
  }
}

template <class T>
__global__ void k_gather_in(int n, const int32_t *__restrict__ n2o, const double *__restrict__ src,
                            T *__restrict__ dst, double shift) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = static_cast<T>(src[n2o[i]] - shift);
}

// scatter back to reference order; bit 1 of *flags marks a NaN/Inf value
template <class T>
__global__ void k_scatter_out(int n, const int32_t *__restrict__ n2o, const T *__restrict__ src,
                              double *__restrict__ dst, double shift, int *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double v = static_cast<double>(src[i]) + shift;
    dst[n2o[i]] = v;
    if (flags && !isfinite(v)) atomicOr(flags, 2);
  }
}

// j runs over the reference order, so that the host array is read (or
// written) in order; the device side takes the permutation
template <class T>
__global__ void k_load_host(int n, const int32_t *__restrict__ o2n,
                            const double *__restrict__ src, T *__restrict__ yn,
                            T *__restrict__ ya, T *__restrict__ ck, double shift) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const T v = static_cast<T>(src[j] - shift);
    const int i = o2n[j];
    yn[i] = v;
    ya[i] = v;
    if (ck) ck[i] = v;
  }
}

template <class T>
__global__ void k_store_host(int n, const int32_t *__restrict__ o2n, const T *__restrict__ src,
                             double *__restrict__ dst, double shift, int *flags) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) {
    const double v = static_cast<double>(src[o2n[j]]) + shift;
    dst[j] = v;
    if (!isfinite(v)) atomicOr(flags, 2);
  }
}

// vecrecon_trsk_tg, interpack.f90:3852-3976 (var%pos == 6)
__global__ void k_trsk_tangent(DevMesh M, const double *__restrict__ u, double *__restrict__ utg) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const int ns = M.e_nst[e];
  double t = 0.0;
  for (int s = 0; s < ns; ++s) {
    const int k = M.e_stk[s * ne + e];
    t = t + u[k] * M.e_dleng[k] * M.e_stw[s * ne + e];
  }
  utg[e] = -t / M.e_leng[e];
}

// ---- compensated summation (Neumaier) -------------------------------------
struct KSum {
  double s, c;
  __device__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x))
      c = c + ((s - t) + x);
    else
      c = c + ((x - t) + s);
    s = t;
  }
  __device__ void merge(const KSum &o) {
    add(o.s);
    c = c + o.c;
  }
};

template <int NQ>
__device__ void block_reduce_store(KSum (&acc)[NQ], double *__restrict__ scratch) {
  // warp level: plain sums of the sums and of the compensations (32 terms,
  // error ~1e-15 relative; FP64 operations are slow on this GPU, and a
  // Neumaier merge costs four times a plain add)
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    for (int off = 16; off > 0; off >>= 1) {
      acc[q].s += __shfl_down_sync(0xffffffffu, acc[q].s, off);
      acc[q].c += __shfl_down_sync(0xffffffffu, acc[q].c, off);
    }
  }
  __shared__ double sh[kRedThreads / 32][NQ][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      sh[warp][q][0] = acc[q].s;
      sh[warp][q][1] = acc[q].c;
    }
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int q = threadIdx.x;
    KSum t{0.0, 0.0};
    for (int w = 0; w < kRedThreads / 32; ++w) {
      KSum o{sh[w][q][0], sh[w][q][1]};
      t.merge(o);
    }
    scratch[(q * gridDim.x + blockIdx.x) * 2] = t.s;
    scratch[(q * gridDim.x + blockIdx.x) * 2 + 1] = t.c;
  }
}

// one block: quantity q summed over nblk partials; "max" quantities use max
__global__ void k_finalize(const double *__restrict__ scratch, int nblk, int nq,
                           unsigned maxmask, double *__restrict__ result) {
  // one block per quantity; the partials are combined as a tree (a few
  // dependent compensated merges per thread, then 5 shuffle levels per warp
  // and 3 across the warps) rather than by one thread in a row: FP64
  // operations have a long latency on this GPU
  const int q = blockIdx.x;
  if (q >= nq) return;
  static_assert(kRedThreads == 256, "8 warps per block");
  __shared__ double ss[8], sc[8];
  const bool is_max = (maxmask >> q) & 1u;
  KSum a{0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    const double s = scratch[(q * nblk + b) * 2], c = scratch[(q * nblk + b) * 2 + 1];
    if (is_max) {
      a.s = fmax(a.s, s);
    } else {
      KSum o{s, c};
      a.merge(o);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int level = 0; level < 2; ++level) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      KSum o{__shfl_down_sync(0xffffffffu, a.s, off), __shfl_down_sync(0xffffffffu, a.c, off)};
      if (is_max)
        a.s = fmax(a.s, o.s);
      else
        a.merge(o);
    }
    if (level == 1) break;
    if (lane == 0) {
      ss[warp] = a.s;
      sc[warp] = a.c;
    }
    __syncthreads();
    if (warp != 0) return;
    a = lane < 8 ? KSum{ss[lane], sc[lane]} : KSum{0.0, 0.0};
  }
  if (threadIdx.x == 0) result[q] = is_max ? a.s : a.s + a.c;
}

// a / b for the diagnostics: FP64 division is slow on GB300's FP64 pipe, so
// the reciprocal starts from the FP32 one (relative error < 2^-22) and takes
// two Newton-Raphson steps r <- r (2 - b r), which square the error each
// (< 2^-44, then below FP64 rounding); b must be a normal FP32-range number
// (areas, depths)
__device__ __forceinline__ double diag_div(double a, double b) {
  double r = static_cast<double>(__frcp_rn(static_cast<float>(b)));
  r = r * (2.0 - b * r);
  r = r * (2.0 - b * r);
  return a * r;
}

// calc_energies (swm.f90:2686-2752), sumf_areas (:3394), potential enstrophy,
// RMS divergence of the last stage input (hs, us), NaN scan.  FULL = false
// computes the two energies only (the learned correction's drift guard).
// Each thread sums its few dozen terms in plain FP64 (relative error ~1e-14);
// threads, warps, blocks and the grid are combined with Neumaier-compensated
// sums.
template <class T, bool FULL>
__global__ void __launch_bounds__(kRedThreads) k_diag(DevMesh M, const T *__restrict__ h,
                                                      const T *__restrict__ u,
                                                      const T *__restrict__ hs,
                                                      const T *__restrict__ us,
                                                      double h_ref,
                                                      double *__restrict__ scratch) {
  double part[kDiagQ];
#pragma unroll
  for (int q = 0; q < kDiagQ; ++q) part[q] = 0.0;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const double g = M.grav, erad = M.erad;
  double maxdiv = 0.0, umax = 0.0;
  double nan = 0.0;
  if (!FULL) {
    // energies for the learned correction's drift check: terms and each
    // thread's few dozen-term sums in FP32 (the check compares with a value
    // computed the same way, against a bound of 1e-3; FP64 operations are
    // slow on this GPU), the thread sums merged in FP64
    // (FP32 handles read FP32 copies of the weights: even the conversions
    // from FP64 would load the FP64 pipe)
    constexpr bool f32 = sizeof(T) == sizeof(float);
    const float gf = static_cast<float>(g), hr = static_cast<float>(h_ref);
    float pe = 0.0f, ke = 0.0f, um = 0.0f;
    for (int i = tid; i < M.nv; i += stride) {
      const float hi = static_cast<float>(h[i]) + hr;
      if (!isfinite(hi)) nan = 1.0;
      const float A = f32 ? M.c_area32[i] : static_cast<float>(M.c_areag[i]);
      const float b = f32 ? M.c_bt32[i] : static_cast<float>(M.c_bt[i]);
      pe += A * gf * hi * (hi * 0.5f + b);
    }
    for (int e = tid; e < M.ne; e += stride) {
      const float ue = static_cast<float>(u[e]);
      if (!isfinite(ue)) nan = 1.0;
      um = fmaxf(um, fabsf(ue));
      const float he = (static_cast<float>(hs[M.e_v[e]]) +
                        static_cast<float>(hs[M.e_v[M.ne + e]])) * 0.5f + hr;
      const float Ae = f32 ? M.e_area32[e] : static_cast<float>(M.e_area[e]);
      ke += Ae * he * (ue * ue);
    }
    // warp sums in FP32, the block's warps in FP64; the other quantities'
    // partials are zero
    float ne = nan;
    for (int off = 16; off > 0; off >>= 1) {
      pe += __shfl_down_sync(0xffffffffu, pe, off);
      ke += __shfl_down_sync(0xffffffffu, ke, off);
      um = fmaxf(um, __shfl_down_sync(0xffffffffu, um, off));
      ne = fmaxf(ne, __shfl_down_sync(0xffffffffu, ne, off));
    }
    __shared__ float se[4][kRedThreads / 32];
    const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (ln == 0) {
      se[0][wp] = pe;
      se[1][wp] = ke;
      se[2][wp] = um;
      se[3][wp] = ne;
    }
    __syncthreads();
    if (threadIdx.x < kDiagQ) {
      const int q = threadIdx.x;
      double v = 0.0;
      for (int w = 0; w < kRedThreads / 32; ++w) {
        if (q == Q_PE) v += static_cast<double>(se[0][w]);
        if (q == Q_KE) v += static_cast<double>(se[1][w]);
        if (q == Q_UMAX) v = fmax(v, static_cast<double>(se[2][w]));
        if (q == Q_NAN) v = fmax(v, static_cast<double>(se[3][w]));
      }
      scratch[(q * gridDim.x + blockIdx.x) * 2] = v;
      scratch[(q * gridDim.x + blockIdx.x) * 2 + 1] = 0.0;
    }
    return;
  }
  for (int i = tid; FULL && i < M.nv; i += stride) {
    const double A = M.c_areag[i];
    const double hi = static_cast<double>(h[i]) + h_ref;
    const double b = M.c_bt[i];
    if (!isfinite(hi)) nan = 1.0;
    part[Q_PE] += A * g * hi * (hi * 0.5 + b);
    part[Q_AREA] += A;
    part[Q_AH] += A * hi;
    part[Q_AHB] += A * (hi + b);
    part[Q_AB2] += A * b * b;
    // div_hx(u) of the last stage input (diagnostic in tendency, :2570)
    const int n = M.c_nnb[i];
    double d = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = M.c_ed[j * M.nv + i];
      d = d + static_cast<double>(us[e]) * M.c_sd[j * M.nv + i];
    }
    d = diag_div(d, A * erad);
    part[Q_ADIV2] += A * (d * d);
    maxdiv = fmax(maxdiv, fabs(d));
  }
  for (int e = tid; FULL && e < M.ne; e += stride) {
    const double ue = static_cast<double>(u[e]);
    if (!isfinite(ue)) nan = 1.0;
    umax = fmax(umax, fabs(ue));
    // h_ed of the last stage input, as calc_energies uses (swm.f90:2738)
    const double he =
        (static_cast<double>(hs[M.e_v[e]]) + static_cast<double>(hs[M.e_v[M.ne + e]])) * 0.5 + h_ref;
    part[Q_KE] += M.e_area[e] * he * (ue * ue);
  }
  for (int t = tid; FULL && t < M.nt; t += stride) {
    double eta = 0.0, ht = 0.0;
    for (int s = 0; s < 3; ++s) {
      eta = eta + static_cast<double>(us[M.t_ed[s * M.nt + t]]) * M.t_lt[s * M.nt + t];
      ht = ht + M.t_kite[s * M.nt + t] * (static_cast<double>(hs[M.t_v[s * M.nt + t]]) + h_ref);
    }
    const double A = M.t_areag[t];
    eta = diag_div(eta, A * erad);
    eta = eta + M.t_f[t];
    ht = diag_div(ht, A);
    const double q = ht != 0.0 ? diag_div(eta, ht) : 0.0;
    part[Q_ENS] += A * ht * (q * q) * 0.5;
  }
  KSum acc[kDiagQ];
#pragma unroll
  for (int q = 0; q < kDiagQ; ++q) acc[q] = KSum{part[q], 0.0};
  // max-type entries are reduced with max, not a sum: pre-reduce them (their
  // sums, all zero, are overwritten below)
  const int kMaxQ[3] = {Q_MAXDIV, Q_NAN, Q_UMAX};
  double mx[3] = {maxdiv, nan, umax};
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int off = 16; off > 0; off >>= 1)
      mx[k] = fmax(mx[k], __shfl_down_sync(0xffffffffu, mx[k], off));
  __shared__ double smax[3][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 3; ++k) smax[k][warp] = mx[k];
  __syncthreads();
  double bm[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 3; ++k)
    for (int w = 0; w < kRedThreads / 32; ++w) bm[k] = fmax(bm[k], smax[k][w]);
  block_reduce_store<kDiagQ>(acc, scratch);
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) scratch[(kMaxQ[k] * gridDim.x + blockIdx.x) * 2] = bm[k];
}

// error_calc partials (swm.f90:3492-3543): weights A_i (cells) and l*d/2
// (edges, sumfsq_areas :3468-3474)
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_errors(DevMesh M, const T *__restrict__ h,
                                                        const T *__restrict__ u, double h_ref,
                                                        const double *__restrict__ href,
                                                        const double *__restrict__ uref,
                                                        double *__restrict__ scratch) {
  constexpr int NQ = 8;
  KSum acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = KSum{0.0, 0.0};
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double mdh = 0.0, mrh = 0.0, mdu = 0.0, mru = 0.0;
  for (int i = tid; i < M.nv; i += stride) {
    const double A = M.c_areag[i];
    const double r = href[i];
    const double dif = (static_cast<double>(h[i]) + h_ref) - r;
    acc[0].add(A * (dif * dif));
    acc[1].add(A * (r * r));
    mdh = fmax(mdh, fabs(dif));
    mrh = fmax(mrh, fabs(r));
  }
  for (int e = tid; e < M.ne; e += stride) {
    const double w = M.e_area[e];
    const double r = uref[e];
    const double dif = static_cast<double>(u[e]) - r;
    acc[4].add(w * (dif * dif));
    acc[5].add(w * (r * r));
    mdu = fmax(mdu, fabs(dif));
    mru = fmax(mru, fabs(r));
  }
  double mx[4] = {mdh, mrh, mdu, mru};
  for (int k = 0; k < 4; ++k)
    for (int off = 16; off > 0; off >>= 1) mx[k] = fmax(mx[k], __shfl_down_sync(0xffffffffu, mx[k], off));
  __shared__ double smax[4][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 4; ++k) smax[k][warp] = mx[k];
  __syncthreads();
  double bm[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; ++k)
    for (int w = 0; w < kRedThreads / 32; ++w) bm[k] = fmax(bm[k], smax[k][w]);
  block_reduce_store<NQ>(acc, scratch);
  __syncthreads();
  if (threadIdx.x == 0) {
    scratch[(2 * gridDim.x + blockIdx.x) * 2] = bm[0];
    scratch[(3 * gridDim.x + blockIdx.x) * 2] = bm[1];
    scratch[(6 * gridDim.x + blockIdx.x) * 2] = bm[2];
    scratch[(7 * gridDim.x + blockIdx.x) * 2] = bm[3];
  }
}

inline int nblocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void launch_stage64(const DevMesh &M, const Work<double> &W, const double *h_in,
                    const double *u_in, double *h_out, double *u_out, int stage, double dt,
                    cudaStream_t s, cudaEvent_t *ev) {
  if (ev) cudaEventRecord(ev[0], s);
  // diffusion: the triangle and cell kernels also write K_tr zeta(u) and
  // K div u; the edge gradients follow them (and, with hyperdiffusion, the
  // second application), before the edge kernel
  const Diffusion<double> &D = W.dif;
  const int sch = W.scheme;
  k_tri64<<<nblocks(M.nt, 256), 256, 0, s>>>(M, h_in, u_in, W.q_tr, W.pv_on, W.flags, D.kt,
                                              D.on ? D.coefvort : nullptr, sch, W.eta_t,
                                              W.h_trs);
  if (ev) cudaEventRecord(ev[1], s);
  const Apvm<double> &A = W.apvm;
  if (A.on) {
    const int nbt = nblocks(M.nt, 256);
    k_qgrad64<<<nblocks(M.ne, 256), 256, 0, s>>>(M, W.q_tr, A.qge);
    k_apvm64<<<nbt + nblocks(M.nv, 256), 256, 0, s>>>(M, A.qge, u_in, A.qg, A.vhx, nbt);
  }
  k_edge_pre64<<<nblocks(M.ne, 256), 256, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ed, W.uh, W.q_ed,
                                                   A.on ? A.qg : nullptr, A.vhx, A.coef, sch,
                                                   W.eta_t, W.h_trs, W.pv_on, W.flags);
  if (sch == IMODEL_SWM_DTRED)
    k_vhq64<<<nblocks(M.nt, 256), 256, 0, s>>>(M, W.uh, W.q_tr, W.vhq);
  if (ev) cudaEventRecord(ev[2], s);
  k_cell64<<<nblocks(M.nv, 256), 256, 0, s>>>(M, h_in, u_in, W.uh, W.bern, W.yn_h, W.acc_h,
                                               h_out, W.tend_h, stage, dt, D.kcv,
                                               D.on ? D.coefdiv : nullptr,
                                               sch == IMODEL_SWM_PXT16 ? 1 : 0);
  if (D.on) {
    k_diflap64<<<nblocks(M.ne, 256), 256, 0, s>>>(M, D.coefdiv, D.coefvort, D.lap);
    if (D.k4) {
      const int nbc = nblocks(M.nv, 256), nbt = nblocks(M.nt, 256);
      k_difcv64<<<nbc + nbt, 256, 0, s>>>(M, D.lap, D.kcv, D.kt, D.coefdiv, D.coefvort, nbc);
      k_diflap64<<<nblocks(M.ne, 256), 256, 0, s>>>(M, D.coefdiv, D.coefvort, D.lap2);
    }
  }
  if (ev) cudaEventRecord(ev[3], s);
  if (sch == IMODEL_SWM_PXT16 || sch == IMODEL_SWM_DTRED)
    k_edge64r<<<nblocks(M.ne, 256), 256, 0, s>>>(M, W.bern, W.uh, W.q_ed, W.vhq, W.yn_u, W.acc_u,
                                                  u_out, W.tend_u, stage, dt, W.mom_on,
                                                  D.k2 ? D.lap : nullptr,
                                                  D.k4 ? D.lap2 : nullptr, sch);
  else
    k_edge64<<<nblocks(M.ne, 256), 256, 0, s>>>(M, W.bern, W.uh, W.q_ed, W.yn_u, W.acc_u, u_out,
                                                 W.tend_u, stage, dt, W.mom_on,
                                                 D.k2 ? D.lap : nullptr, D.k4 ? D.lap2 : nullptr,
                                                 sch == IMODEL_SWM_GASS18 ? M.e_stq : nullptr);
  if (ev) cudaEventRecord(ev[4], s);
}

void launch_dif_coefs(const DevMesh &M, const double *kf, double k, bool take_sqrt, double *kc64,
                      float *kc32, double *kt64, float *kt32, cudaStream_t s) {
  const int nbc = nblocks(M.nv, 256);
  k_dif_coefs<<<nbc + nblocks(M.nt, 256), 256, 0, s>>>(M, kf, k, take_sqrt ? 1 : 0, kc64, kc32,
                                                        kt64, kt32, nbc);
}

void launch_gather_in(int n, const int32_t *n2o, const double *src, double *dst, double shift,
                      cudaStream_t s) {
  k_gather_in<double><<<nblocks(n, 256), 256, 0, s>>>(n, n2o, src, dst, shift);
}
void launch_gather_in32(int n, const int32_t *n2o, const double *src, float *dst, double shift,
                        cudaStream_t s) {
  k_gather_in<float><<<nblocks(n, 256), 256, 0, s>>>(n, n2o, src, dst, shift);
}
void launch_scatter_out(int n, const int32_t *n2o, const double *src, double *dst, double shift,
                        int *flags, cudaStream_t s) {
  k_scatter_out<double><<<nblocks(n, 256), 256, 0, s>>>(n, n2o, src, dst, shift, flags);
}
void launch_scatter_out32(int n, const int32_t *n2o, const float *src, double *dst,
                          double shift, int *flags, cudaStream_t s) {
  k_scatter_out<float><<<nblocks(n, 256), 256, 0, s>>>(n, n2o, src, dst, shift, flags);
}

template <class T>
void launch_load_host(int n, const int32_t *o2n, const double *src, T *yn, T *ya, T *ck,
                      double shift, cudaStream_t s) {
  k_load_host<T><<<nblocks(n, 256), 256, 0, s>>>(n, o2n, src, yn, ya, ck, shift);
}
template <class T>
void launch_store_host(int n, const int32_t *o2n, const T *src, double *dst, double shift,
                       int *flags, cudaStream_t s) {
  k_store_host<T><<<nblocks(n, 256), 256, 0, s>>>(n, o2n, src, dst, shift, flags);
}
template void launch_load_host<double>(int, const int32_t *, const double *, double *, double *,
                                       double *, double, cudaStream_t);
template void launch_load_host<float>(int, const int32_t *, const double *, float *, float *,
                                      float *, double, cudaStream_t);
template void launch_store_host<double>(int, const int32_t *, const double *, double *, double,
                                        int *, cudaStream_t);
template void launch_store_host<float>(int, const int32_t *, const float *, double *, double,
                                       int *, cudaStream_t);

void launch_trsk_tangent(const DevMesh &M, const double *u, double *utg, cudaStream_t s) {
  k_trsk_tangent<<<nblocks(M.ne, 256), 256, 0, s>>>(M, u, utg);
}

template <class T>
void launch_diag(const DevMesh &M, const Work<T> &W, const T *h, const T *u, const T *hs,
                 const T *us, double *scratch, double *result, cudaStream_t s,
                 bool energy_only) {
  if (energy_only)
    k_diag<T, false><<<kRedBlocks, kRedThreads, 0, s>>>(M, h, u, hs, us,
                                                         static_cast<double>(W.h_ref), scratch);
  else
    k_diag<T, true><<<kRedBlocks, kRedThreads, 0, s>>>(M, h, u, hs, us,
                                                        static_cast<double>(W.h_ref), scratch);
  const unsigned maxmask = (1u << Q_MAXDIV) | (1u << Q_NAN) | (1u << Q_UMAX);
  k_finalize<<<kDiagQ, kRedThreads, 0, s>>>(scratch, kRedBlocks, kDiagQ, maxmask, result);
}
template void launch_diag<double>(const DevMesh &, const Work<double> &, const double *,
                                  const double *, const double *, const double *, double *,
                                  double *, cudaStream_t, bool);
template void launch_diag<float>(const DevMesh &, const Work<float> &, const float *,
                                 const float *, const float *, const float *, double *,
                                 double *, cudaStream_t, bool);

template <class T>
void launch_errors(const DevMesh &M, const T *h, const T *u, double h_ref, const double *href,
                   const double *uref, double *scratch, double *result, cudaStream_t s) {
  k_errors<T><<<kRedBlocks, kRedThreads, 0, s>>>(M, h, u, h_ref, href, uref, scratch);
  const unsigned maxmask = (1u << 2) | (1u << 3) | (1u << 6) | (1u << 7);
  k_finalize<<<8, kRedThreads, 0, s>>>(scratch, kRedBlocks, 8, maxmask, result);
}
template void launch_errors<double>(const DevMesh &, const double *, const double *, double,
                                    const double *, const double *, double *, double *,
                                    cudaStream_t);
template void launch_errors<float>(const DevMesh &, const float *, const float *, double,
                                   const double *, const double *, double *, double *,
                                   cudaStream_t);

}  // namespace imodel
