// CPU restatement of iModel's TRSK shallow-water time step (FP64).
//
// TEST INFRASTRUCTURE ONLY: the correctness oracle for the GB300 kernels and
// the CPU baseline timed beside them.  Nothing in the product links this.
//
// It follows the Fortran loop by loop for the branches the trsk10, pxt16 and
// gass18 wrappers (and the dtred Coriolis reconstruction), HTC staggering and
// geodesic areas select (swm_data.f90:446-507), with the
// same per-entity accumulation order and one OpenMP parallel loop per
// operator, like the reference's `!$omp parallel do schedule(static)`.
// Build with -ffp-contract=off so no multiply-add is fused.
//
// Parity status: unpinned against the Fortran binary (no Fortran compiler);
// pinned by the reference's known answers (see tests/test_oracle_kat.py).

#include "swm_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

// constants.f90:31, :45 (pi from a float literal; eps = epsilon(1.))
const double kPi = 4.0 * static_cast<double>(0.78539816339744830961566f);
const double kEps = static_cast<double>(1.1920928955078125e-07f);

struct Oracle {
  imodel_swm_mesh m;
  int testcase;
  int nthreads;
  std::vector<double> bt, fcor;
  std::vector<double> h_ed, uh, eta, h_tr, eta_ed, q_tr, q_ed, divuh, ke, hbt, ghbK, grad,
      uhq, divu, zeta, vhx;
  std::vector<double> massf[4], momf[4], h_tmp, u_tmp;
  // diffusion_ed / hyperdiffusion_ed with constant coefficients
  bool k2_on = false, k4_on = false;
  std::vector<double> dif_hx;          // dif_coef_hx [nv]
  std::vector<double> dif_tr, sgtg;    // dif_coef_tr [nt]; grad_ed_tg signcor [ne]
  std::vector<double> coefdiv, coefvort, lapu, lap_lapu, div_lap, vort_lap;
  // apvm (swm_operators.f90:1465-1543): pv_stab = "apvm", pvspar, the run's dt
  bool apvm_on = false;
  double pvspar = 0.0, apvm_dt = 0.0;
  std::vector<double> cc;              // tr%c%p [nt][3]
  std::vector<double> q_grad_ed, q_grad_tr;   // [ne], [nt][3]
  // method wrapper (swm_data.f90:446-507): 0 trsk10, 1 pxt16, 2 gass18,
  // 3 trsk10 with the dtred Coriolis reconstruction (mtdwrapper "none")
  int scheme = 0;
  std::vector<double> bary;            // tr%c%b [nt][3] (pxt16)
  std::vector<double> dist;            // arclen(ed%c, tr(sh(i))%c) [ne][2] (pxt16, dtred)
  std::vector<double> edarea;          // sphtriarea(tr%c, ed%v) [nt][3] (gass18)
  std::vector<int> conn;               // gethxedgeconnection(l, k) per TRSK term [ne][12]
  std::vector<double> h_rhb, vhq_tr;   // [ne] (gass18), [nt][3] (dtred)
  std::vector<double> h_trk;           // kite-weighted h_tr of the last call (diagnostics)
};

#define I6(i, j) (static_cast<size_t>(i) * 6 + (j))

// getedindexonhx, smeshpack.f90:4099-4125 (1-based result, 0 if absent)
inline int getedindexonhx(const imodel_swm_mesh &m, int ed, int cell) {
  for (int i = 0; i < m.nnb[cell]; ++i)
    if (m.v_ed[I6(cell, i)] - 1 == ed) return i + 1;
  return 0;
}

// ---- spherical geometry of smeshpack.f90, as the scheme set-up uses it ----
inline double dot3(const double *a, const double *b) {
  double s = a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}
// cross_product, smeshpack.f90:6560-6578
inline void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
// det, smeshpack.f90:6580-6595
inline double det3(const double *p1, const double *p2, const double *p3) {
  double c[3];
  cross3(p1, p2, c);
  return dot3(c, p3);
}
// arclen, smeshpack.f90:4624-4657
inline double arclen(const double *p, const double *q) {
  const double s[3] = {p[0] + q[0], p[1] + q[1], p[2] + q[2]};
  const double d = dot3(s, s);
  if (d == 0.0) return kPi;
  if (d >= 4.0) return 0.0;
  return 2.0 * std::atan(std::sqrt((4.0 - d) / d));
}
inline double norm3(const double *p) { return std::sqrt(dot3(p, p)); }
// sphtriarea (L'Huilier), smeshpack.f90:4710-4762
double sphtriarea(const double *p1, const double *p2, const double *p3) {
  const double d12[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
  const double d23[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
  const double d13[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
  const double tol = kEps / 100.0;
  if (norm3(d12) < tol || norm3(d23) < tol || norm3(d13) < tol) return 0.0;
  const double a = arclen(p1, p2), b = arclen(p2, p3), c = arclen(p3, p1);
  const double s = (a + b + c) / 2.0;
  double t = std::tan(s / 2.0) * std::tan((s - a) / 2.0);
  t = t * std::tan((s - b) / 2.0);
  t = t * std::tan((s - c) / 2.0);
  if (t < 0.0) return 0.0;
  return 4.0 * std::atan(std::sqrt(t));
}
// proj_vec_sphere, smeshpack.f90:4419-4433: v - (v . p) p / |p|
inline void proj_sphere(double *v, const double *p) {
  const double vp = dot3(v, p);
  const double np = norm3(p);
  for (int k = 0; k < 3; ++k) v[k] = v[k] - vp * p[k] / np;
}

// getedgeintriangle + gethxedgeconnection, smeshpack.f90:4127-4244 (0-based
// edges; 0-based third edge, -1 for "equal" (the reference's 0) and -2 for
// "not connected" (its -1))
int edge_connection(const imodel_swm_mesh &m, int ed1, int ed2) {
  if (ed1 == ed2) return -1;
  const int tr1 = m.ed_sh[2 * ed1] - 1, tr2 = m.ed_sh[2 * ed1 + 1] - 1;
  int tr = -1;
  for (int i = 0; i < 3; ++i) {
    if (ed2 == m.tr_ed[3 * tr1 + i] - 1) {
      tr = tr1;
      break;
    }
    if (ed2 == m.tr_ed[3 * tr2 + i] - 1) {
      tr = tr2;
      break;
    }
  }
  if (tr >= 0) {
    for (int i = 0; i < 3; ++i) {
      const int ed = m.tr_ed[3 * tr + i] - 1;
      if (ed != ed1 && ed != ed2) return ed;
    }
  }
  // edhx(edref)%v = ed(edref)%sh: the triangles at the ends of ed2's dual edge
  for (int j = 0; j < 2; ++j) {
    const int trj = m.ed_sh[2 * ed2 + j] - 1;
    for (int i = 0; i < 3; ++i) {
      const int edtmp = m.tr_ed[3 * trj + i] - 1;
      if (edtmp == ed2) continue;
      const int a = m.ed_sh[2 * edtmp] - 1, b = m.ed_sh[2 * edtmp + 1] - 1;
      const int other = a == trj ? b : a;
      for (int l = 0; l < 3; ++l)
        if (ed1 == m.tr_ed[3 * other + l] - 1) return edtmp;
    }
  }
  return -2;
}

// diffusion_ed (swm_operators.f90:855-895): coef*div and coef*vort
// (scalar_elem_product), grad_ed of the first (:511-548, HTC), grad_ed_tg of
// the second (:738-777, HTC), lap = difference
void diffusion(Oracle &o, const double *div, const double *vort, double *lap) {
  const imodel_swm_mesh &m = o.m;
  const int nv = m.nv, ne = m.ne, nt = m.nt;
  const double erad = m.erad;
  const int nth = o.nthreads;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) o.coefdiv[i] = o.dif_hx[i] * div[i];
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int k = 0; k < nt; ++k) o.coefvort[k] = o.dif_tr[k] * vort[k];
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) {
    double g = o.coefdiv[m.ed_v[2 * l + 1] - 1] - o.coefdiv[m.ed_v[2 * l] - 1];
    g = g / m.ed_leng[l] / erad;
    const int k1 = m.ed_sh[2 * l] - 1, k2 = m.ed_sh[2 * l + 1] - 1;
    double gt = o.sgtg[l] * (o.coefvort[k2] - o.coefvort[k1]);
    gt = gt / (m.edhx_leng[l] * erad);
    lap[l] = g - gt;
  }
}

// scalar_tr2ed (swm_operators.f90:124-176), HTC: the plain average for
// trsk interpolation, rhombus (triangle-area) weights for gass, and
// circumcentre-distance weights for bary
void tr2ed(Oracle &o, const double *ftr, double *fed) {
  const imodel_swm_mesh &m = o.m;
  const int ne = m.ne;
  const int nth = o.nthreads;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) {
    const int k1 = m.ed_sh[2 * l] - 1, k2 = m.ed_sh[2 * l + 1] - 1;
    if (o.scheme == 0 || o.scheme == 3) {
      fed[l] = 0.5 * (ftr[k1] + ftr[k2]);
    } else if (o.scheme == 2) {
      const double a1 = m.tr_areag[k1], a2 = m.tr_areag[k2];
      fed[l] = (a1 * ftr[k1] + a2 * ftr[k2]) / (a1 + a2);
    } else {
      const double d1 = o.dist[2 * static_cast<size_t>(l)], d2 = o.dist[2 * static_cast<size_t>(l) + 1];
      fed[l] = (d2 * ftr[k1] + d1 * ftr[k2]) / (d1 + d2);
    }
  }
}

// tendency, swm.f90:2416-2598
int tendency(Oracle &o, const double *h, const double *u, double *masseq, double *momeq) {
  const imodel_swm_mesh &m = o.m;
  const int nv = m.nv, ne = m.ne, nt = m.nt;
  const double erad = m.erad, grav = m.grav;
  int nth = o.nthreads;
  // zero_vector x2 (swm_operators.f90:1652)
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) momeq[l] = 0.0;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) masseq[i] = 0.0;

  // scalar_hx2ed (swm_operators.f90:89-97) and scalar_elem_product (:1546)
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l)
    o.h_ed[l] = (h[m.ed_v[2 * l] - 1] + h[m.ed_v[2 * l + 1] - 1]) * 0.5;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) o.uh[l] = u[l] * o.h_ed[l];

  // vort_tr (swm_operators.f90:551-611), HTC branch, fsphere=0
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int k = 0; k < nt; ++k) {
    double e = 0.0;
    for (int l = 0; l < 3; ++l) {
      int ed = m.tr_ed[3 * k + l] - 1;
      double signcor = static_cast<double>(m.tr_tg[3 * k + l]);
      e = e + u[ed] * m.ed_leng[ed] * signcor;
    }
    e = e / m.tr_areag[k] / erad;
    e = e + o.fcor[k];
    o.eta[k] = e;
  }

  // depth at the triangles (swm.f90:2459-2464): scalar_hx2tr
  // (swm_operators.f90:229-284), trsk branch (kite areas) or bary branch
  // (barycentric coordinates of the circumcentre); gass: scalar_edtr2trcc
  // (:286-343, geodesic areas) of h_ed, and its rhombus average h_rhb
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int k = 0; k < nt; ++k) {
    double f = 0.0;
    for (int i = 0; i < 3; ++i) f = f + m.tr_trhx_area[3 * k + i] * h[m.tr_v[3 * k + i] - 1];
    f = f / m.tr_areag[k];
    if (o.scheme == 0 || o.scheme == 3) {
      o.h_tr[k] = f;
    } else {
      o.h_trk[k] = f;
      double g = 0.0;
      if (o.scheme == 1) {
        for (int i = 0; i < 3; ++i) g = g + o.bary[3 * k + i] * h[m.tr_v[3 * k + i] - 1];
      } else {
        for (int i = 0; i < 3; ++i) g = g + o.edarea[3 * k + i] * o.h_ed[m.tr_ed[3 * k + i] - 1];
        g = g / m.tr_areag[k];
      }
      o.h_tr[k] = g;
    }
  }
  if (o.scheme == 2) tr2ed(o, o.h_tr.data(), o.h_rhb.data());

  // scalar_tr2ed(eta -> eta_ed) (swm_operators.f90:124-176)
  tr2ed(o, o.eta.data(), o.eta_ed.data());

  // scalar_elem_divide (swm_operators.f90:1579-1615)
  int divzero = 0;
  if (o.testcase < 2) {
    for (int k = 0; k < nt; ++k) o.q_tr[k] = 0.0;
  } else {
#pragma omp parallel for schedule(static) num_threads(nth) reduction(+ : divzero)
    for (int k = 0; k < nt; ++k) {
      if (std::fabs(o.h_tr[k]) < kEps / 100000.0)
        divzero += 1;
      else
        o.q_tr[k] = o.eta[k] / o.h_tr[k];
    }
  }
  if (divzero) return IMODEL_SWM_EDIVZERO;

  // PV at the edges (swm.f90:2475-2480): scalar_tr2ed(q_tr), or for gass
  // scalar_elem_divide(eta_ed, h_rhb) with its division guard
  if (o.scheme == 2) {
    if (o.testcase < 2) {
      for (int l = 0; l < ne; ++l) o.q_ed[l] = 0.0;
    } else {
#pragma omp parallel for schedule(static) num_threads(nth) reduction(+ : divzero)
      for (int l = 0; l < ne; ++l) {
        if (std::fabs(o.h_rhb[l]) < kEps / 100000.0)
          divzero += 1;
        else
          o.q_ed[l] = o.eta_ed[l] / o.h_rhb[l];
      }
    }
    if (divzero) return IMODEL_SWM_EDIVZERO;
  } else {
    tr2ed(o, o.q_tr.data(), o.q_ed.data());
  }

  // dtred: vector_edhx2tr_perot(uh -> vhq_tr) (swm_operators.f90:345-406,
  // HTC), times q_tr (vector_elem_product, :1617-1649)
  if (o.scheme == 3) {
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int k = 0; k < nt; ++k) {
      const double *c = &o.cc[3 * static_cast<size_t>(k)];
      double v[3] = {0.0, 0.0, 0.0};
      for (int l = 0; l < 3; ++l) {
        const int ed = m.tr_ed[3 * k + l] - 1;
        const double signcor = std::copysign(1.0, static_cast<double>(m.tr_tg[3 * k + l]));
        const double *ec = m.ed_c + 3 * static_cast<size_t>(ed);
        for (int i = 0; i < 3; ++i)
          v[i] = v[i] + signcor * o.uh[ed] * (ec[i] - c[i]) * m.ed_leng[ed];
      }
      double w[3];
      cross3(c, v, w);
      for (int i = 0; i < 3; ++i)
        o.vhq_tr[3 * static_cast<size_t>(k) + i] = w[i] / m.tr_areag[k] * o.q_tr[k];
    }
  }

  // vector_edhx2hx_perot(u -> v_hx) (swm_operators.f90:454-509): computed by
  // the reference on every call although trsk10 never reads it.
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    const double *p = m.v_p + 3 * static_cast<size_t>(i);
    for (int l = 0; l < m.nnb[i]; ++l) {
      int ed = m.v_ed[I6(i, l)] - 1;
      double signcor = static_cast<double>(m.hx_ttgout[I6(i, l)]);
      const double *c = m.ed_c + 3 * static_cast<size_t>(ed);
      double s = signcor * u[ed];
      v0 = v0 + s * (c[0] - p[0]) * m.edhx_leng[ed];
      v1 = v1 + s * (c[1] - p[1]) * m.edhx_leng[ed];
      v2 = v2 + s * (c[2] - p[2]) * m.edhx_leng[ed];
    }
    v0 = v0 / m.hx_areag[i];
    v1 = v1 / m.hx_areag[i];
    v2 = v2 / m.hx_areag[i];
    double vp = v0 * p[0] + v1 * p[1] + v2 * p[2];
    double np = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    o.vhx[3 * static_cast<size_t>(i)] = v0 - vp * p[0] / np;
    o.vhx[3 * static_cast<size_t>(i) + 1] = v1 - vp * p[1] / np;
    o.vhx[3 * static_cast<size_t>(i) + 2] = v2 - vp * p[2] / np;
  }

  if (o.apvm_on) {
    // grad_tr2ed(q_tr -> q_grad_ed) (swm_operators.f90:1427-1463)
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int l = 0; l < ne; ++l) {
      const int k1 = m.ed_sh[2 * l] - 1, k2 = m.ed_sh[2 * l + 1] - 1;
      o.q_grad_ed[l] = o.sgtg[l] * (o.q_tr[k2] - o.q_tr[k1]) / m.edhx_leng[l] / erad;
    }
    // vector_edtr2tr_perot(q_grad_ed -> q_grad_tr) (:408-452);
    // dsign(1, tr%nr) with tr%nr = -tr%tg (smeshpack.f90:853-859)
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int k = 0; k < nt; ++k) {
      const double *c = &o.cc[3 * static_cast<size_t>(k)];
      double v0 = 0.0, v1 = 0.0, v2 = 0.0;
      for (int l = 0; l < 3; ++l) {
        const int ed = m.tr_ed[3 * k + l] - 1;
        const double signcor = -static_cast<double>(m.tr_tg[3 * k + l]);
        const double *ec = m.ed_c + 3 * static_cast<size_t>(ed);
        const double s = signcor * o.q_grad_ed[ed];
        v0 = v0 + s * (ec[0] - c[0]) * m.ed_leng[ed];
        v1 = v1 + s * (ec[1] - c[1]) * m.ed_leng[ed];
        v2 = v2 + s * (ec[2] - c[2]) * m.ed_leng[ed];
      }
      v0 = v0 / m.tr_areag[k];
      v1 = v1 / m.tr_areag[k];
      v2 = v2 / m.tr_areag[k];
      // proj_vec_sphere (smeshpack.f90:4419-4433)
      const double vp = v0 * c[0] + v1 * c[1] + v2 * c[2];
      const double nc = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      o.q_grad_tr[3 * static_cast<size_t>(k)] = v0 - vp * c[0] / nc;
      o.q_grad_tr[3 * static_cast<size_t>(k) + 1] = v1 - vp * c[1] / nc;
      o.q_grad_tr[3 * static_cast<size_t>(k) + 2] = v2 - vp * c[2] / nc;
    }
    // apvm: q_ed = q_ed - pvspar*dt*(g(sh1) + g(sh2)) . (v(v1) + v(v2))
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int l = 0; l < ne; ++l) {
      const double *g1 = &o.q_grad_tr[3 * static_cast<size_t>(m.ed_sh[2 * l] - 1)];
      const double *g2 = &o.q_grad_tr[3 * static_cast<size_t>(m.ed_sh[2 * l + 1] - 1)];
      const double *w1 = &o.vhx[3 * static_cast<size_t>(m.ed_v[2 * l] - 1)];
      const double *w2 = &o.vhx[3 * static_cast<size_t>(m.ed_v[2 * l + 1] - 1)];
      double d = 0.0;
      for (int k = 0; k < 3; ++k) d = d + (g1[k] + g2[k]) * (w1[k] + w2[k]);
      o.q_ed[l] = o.q_ed[l] - o.pvspar * o.apvm_dt * d;
    }
  }

  // div_hx(uh -> divuh) (swm_operators.f90:613-661), HTC: signcor = ttgout
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    double d = 0.0;
    for (int j = 0; j < m.nnb[i]; ++j) {
      int l = m.v_ed[I6(i, j)] - 1;
      double signcor = static_cast<double>(m.hx_ttgout[I6(i, j)]);
      d = d + signcor * o.uh[l] * m.edhx_leng[l];
    }
    o.divuh[i] = d / m.hx_areag[i] / erad;
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) masseq[i] = -o.divuh[i];

  // kinetic_energy_hx (swm_operators.f90:1132-1217): perhx branch for
  // pxt16 (half the squared Perot velocity), trsk branch otherwise
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    if (o.scheme == 1) {
      const double *v = &o.vhx[3 * static_cast<size_t>(i)];
      o.ke[i] = dot3(v, v) / 2.0;
      continue;
    }
    double k = 0.0, cell_area = 0.0;
    for (int l = 0; l < m.nnb[i]; ++l) {
      int ed = m.v_ed[I6(i, l)] - 1;
      double ed_area = 0.25 * m.ed_leng[ed] * m.edhx_leng[ed];
      cell_area = cell_area + ed_area;
      k = k + ed_area * (u[ed] * u[ed]);
    }
    o.ke[i] = k / cell_area;
  }

  // hbt = h + bt ; ghbK = grav*hbt + ke (swm.f90:2533-2536)
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    o.hbt[i] = h[i] + o.bt[i];
    o.ghbK[i] = grav * o.hbt[i] + o.ke[i];
  }

  // grad_ed, HTC (swm_operators.f90:511-548) ; momeq = -grad
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) {
    double g = o.ghbK[m.ed_v[2 * l + 1] - 1] - o.ghbK[m.ed_v[2 * l] - 1];
    g = g / m.ed_leng[l] / erad;
    o.grad[l] = g;
    momeq[l] = -g;
  }

  // coriolis_ed (swm_operators.f90:1219-1414), HTC: TRSK branch (:1283-1308),
  // its gass variant with the PV of the connecting edge (:1378-1410), the
  // dtred branch (:1310-1329) and the pered branch (:1330-1377)
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) {
    if (o.scheme == 3) {
      const int k1 = m.ed_sh[2 * l] - 1, k2 = m.ed_sh[2 * l + 1] - 1;
      const double d1 = o.dist[2 * static_cast<size_t>(l)], d2 = o.dist[2 * static_cast<size_t>(l) + 1];
      double v[3];
      for (int i = 0; i < 3; ++i)
        v[i] = (d2 * o.vhq_tr[3 * static_cast<size_t>(k1) + i] +
                d1 * o.vhq_tr[3 * static_cast<size_t>(k2) + i]) / (d1 + d2);
      proj_sphere(v, m.ed_c + 3 * static_cast<size_t>(l));
      o.uhq[l] = -dot3(v, m.ed_nr + 3 * static_cast<size_t>(l));
      continue;
    }
    if (o.scheme == 1) {
      double vc[2][3];
      for (int i = 0; i < 2; ++i) {
        const int node = m.ed_v[2 * l + i] - 1;
        const double *p = m.v_p + 3 * static_cast<size_t>(node);
        double v[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < m.nnb[node]; ++j) {
          const int l2 = m.v_ed[I6(node, j)] - 1;
          const double qtmp = 0.5 * (o.q_ed[l] + o.q_ed[l2]);
          const double signcor = static_cast<double>(m.hx_ttgout[I6(node, j)]);
          const double *ec = m.ed_c + 3 * static_cast<size_t>(l2);
          for (int k = 0; k < 3; ++k)
            v[k] = v[k] + signcor * o.uh[l2] * qtmp * (ec[k] - p[k]) * m.edhx_leng[l2];
        }
        for (int k = 0; k < 3; ++k) v[k] = v[k] / m.hx_areag[node];
        proj_sphere(v, p);
        for (int k = 0; k < 3; ++k) vc[i][k] = v[k];
      }
      double v[3];
      for (int k = 0; k < 3; ++k) v[k] = 0.5 * vc[0][k] + 0.5 * vc[1][k];
      proj_sphere(v, m.ed_c + 3 * static_cast<size_t>(l));
      o.uhq[l] = -dot3(v, m.ed_nr + 3 * static_cast<size_t>(l));
      continue;
    }
    double q = 0.0;
    for (int i = 0; i < 2; ++i) {
      int node = m.ed_v[2 * l + i] - 1;
      int edcelli = getedindexonhx(m, l, node);
      for (int j = 0; j < m.nnb[node]; ++j) {
        int k = m.v_ed[I6(node, j)] - 1;
        double signcor = std::copysign(
            1.0, 1.0 * m.hx_ttgout[I6(node, j)] * m.hx_tnrccw[I6(node, edcelli - 1)]);
        double qtmp = 0.5 * (o.q_ed[l] + o.q_ed[k]);
        if (o.scheme == 2) {
          const int ed3 = o.conn[12 * static_cast<size_t>(l) + 6 * i + j];
          if (ed3 >= 0) qtmp = o.q_ed[ed3];
        }
        double w = m.hx_trskw[static_cast<size_t>(node) * 36 + static_cast<size_t>(j) * 6 +
                              (edcelli - 1)];
        q = q + o.uh[k] * qtmp * m.edhx_leng[k] * w * signcor;
      }
    }
    o.uhq[l] = q / m.ed_leng[l];
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) momeq[l] = momeq[l] - o.uhq[l];

  // div_hx(u -> divu) and rel_vort_tr(u -> zeta): diagnostics, every call
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    double d = 0.0;
    for (int j = 0; j < m.nnb[i]; ++j) {
      int l = m.v_ed[I6(i, j)] - 1;
      double signcor = static_cast<double>(m.hx_ttgout[I6(i, j)]);
      d = d + signcor * u[l] * m.edhx_leng[l];
    }
    o.divu[i] = d / m.hx_areag[i] / erad;
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int k = 0; k < nt; ++k) {
    double z = 0.0;
    for (int l = 0; l < 3; ++l) {
      int ed = m.tr_ed[3 * k + l] - 1;
      z = z + u[ed] * m.ed_leng[ed] * static_cast<double>(m.tr_tg[3 * k + l]);
    }
    o.zeta[k] = z / m.tr_areag[k] / erad;
  }

  // Diffusion (swm.f90:2578-2581), hyperdiffusion (:2586-2589)
  if (o.k2_on || o.k4_on) {
    // diffusion_ed (swm_operators.f90:855-895) of u, from divu and zeta
    diffusion(o, o.divu.data(), o.zeta.data(), o.lapu.data());
    if (o.k2_on) {
#pragma omp parallel for schedule(static) num_threads(nth)
      for (int l = 0; l < ne; ++l) momeq[l] = momeq[l] + o.lapu[l];
    }
    if (o.k4_on) {
      // hyperdiffusion_ed (:930-975): div_hx and rel_vort_tr of lapu, then
      // diffusion_ed of them
#pragma omp parallel for schedule(static) num_threads(nth)
      for (int i = 0; i < nv; ++i) {
        double d = 0.0;
        for (int j = 0; j < m.nnb[i]; ++j) {
          int l = m.v_ed[I6(i, j)] - 1;
          double signcor = static_cast<double>(m.hx_ttgout[I6(i, j)]);
          d = d + signcor * o.lapu[l] * m.edhx_leng[l];
        }
        o.div_lap[i] = d / m.hx_areag[i] / erad;
      }
#pragma omp parallel for schedule(static) num_threads(nth)
      for (int k = 0; k < nt; ++k) {
        double z = 0.0;
        for (int l = 0; l < 3; ++l) {
          int ed = m.tr_ed[3 * k + l] - 1;
          z = z + o.lapu[ed] * m.ed_leng[ed] * static_cast<double>(m.tr_tg[3 * k + l]);
        }
        o.vort_lap[k] = z / m.tr_areag[k] / erad;
      }
      diffusion(o, o.div_lap.data(), o.vort_lap.data(), o.lap_lapu.data());
#pragma omp parallel for schedule(static) num_threads(nth)
      for (int l = 0; l < ne; ++l) momeq[l] = momeq[l] - o.lap_lapu[l];
    }
  }

  if (o.testcase <= 1) {
    for (int l = 0; l < ne; ++l) momeq[l] = 0.0;
  }
  return IMODEL_SWM_OK;
}

// ode_rk4, swm.f90:2600-2683
int rk4(Oracle &o, const double *h, const double *u, double *h_new, double *u_new, double dt) {
  const int nv = o.m.nv, ne = o.m.ne;
  int nth = o.nthreads;
  int rc = tendency(o, h, u, o.massf[0].data(), o.momf[0].data());
  if (rc) return rc;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) u_new[l] = u[l] + dt * o.momf[0][l] / 2.0;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) h_new[i] = h[i] + dt * o.massf[0][i] / 2.0;
  rc = tendency(o, h_new, u_new, o.massf[1].data(), o.momf[1].data());
  if (rc) return rc;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) u_new[l] = u[l] + dt * o.momf[1][l] / 2.0;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) h_new[i] = h[i] + dt * o.massf[1][i] / 2.0;
  rc = tendency(o, h_new, u_new, o.massf[2].data(), o.momf[2].data());
  if (rc) return rc;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) u_new[l] = u[l] + dt * o.momf[2][l];
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) h_new[i] = h[i] + dt * o.massf[2][i];
  rc = tendency(o, h_new, u_new, o.massf[3].data(), o.momf[3].data());
  if (rc) return rc;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l)
    u_new[l] = u[l] + dt * (o.momf[0][l] + 2.0 * o.momf[1][l] + 2.0 * o.momf[2][l] +
                            o.momf[3][l]) / 6.0;
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i)
    h_new[i] = h[i] + dt * (o.massf[0][i] + 2.0 * o.massf[1][i] + 2.0 * o.massf[2][i] +
                            o.massf[3][i]) / 6.0;
  return IMODEL_SWM_OK;
}

// sumf_areas / sumfsq_areas, swm.f90:3394-3490 (pos 0: cells, 1: triangles,
// 6: HTC edges; the edge branch of sumf_areas uses hx%areag, as the
// reference does)
double sumfsq_areas(const imodel_swm_mesh &m, const double *f, int pos) {
  double s = 0.0, a = 0.0;
  if (pos == 0) {
    for (int i = 0; i < m.nv; ++i) {
      a = a + m.hx_areag[i];
      s = s + m.hx_areag[i] * (f[i] * f[i]);
    }
  } else if (pos == 1) {
    for (int i = 0; i < m.nt; ++i) {
      a = a + m.tr_areag[i];
      s = s + m.tr_areag[i] * (f[i] * f[i]);
    }
  } else {
    for (int i = 0; i < m.ne; ++i) {
      double area = m.ed_leng[i] * m.edhx_leng[i] * 0.5;
      a = a + area;
      s = s + area * (f[i] * f[i]);
    }
  }
  return s / a;
}

double sumf_areas_cells(const imodel_swm_mesh &m, const double *f) {
  double s = 0.0, a = 0.0;
  for (int i = 0; i < m.nv; ++i) {
    a = a + m.hx_areag[i];
    s = s + m.hx_areag[i] * f[i];
  }
  return s / a;
}

}  // namespace

extern "C" {

void *oracle_create(const imodel_swm_mesh *m, int32_t testcase, const double *bt,
                    int32_t nthreads) {
  if (!m) return nullptr;
  Oracle *o = new Oracle();
  o->m = *m;
  o->testcase = testcase;
  o->nthreads = nthreads > 0 ? nthreads : 1;
  const size_t nv = m->nv, ne = m->ne, nt = m->nt;
  o->bt.assign(nv, 0.0);
  if (bt) std::memcpy(o->bt.data(), bt, nv * sizeof(double));
  o->fcor.resize(nt);
  for (size_t k = 0; k < nt; ++k) o->fcor[k] = 2.0 * m->omega * std::sin(m->tr_c_lat[k]);
  for (auto *v : {&o->h_ed, &o->uh, &o->eta_ed, &o->q_ed, &o->grad, &o->uhq}) v->assign(ne, 0.0);
  for (auto *v : {&o->eta, &o->h_tr, &o->q_tr, &o->zeta}) v->assign(nt, 0.0);
  for (auto *v : {&o->divuh, &o->ke, &o->hbt, &o->ghbK, &o->divu}) v->assign(nv, 0.0);
  o->vhx.assign(3 * nv, 0.0);
  for (int s = 0; s < 4; ++s) {
    o->massf[s].assign(nv, 0.0);
    o->momf[s].assign(ne, 0.0);
  }
  o->h_tmp.assign(nv, 0.0);
  o->u_tmp.assign(ne, 0.0);
  return o;
}

void oracle_destroy(void *o) { delete static_cast<Oracle *>(o); }

// tr%c%p as the unit normal of the triangle's vertex plane, on their side,
// and grad_ed_tg's / grad_tr2ed's sign of ed%nr . (c2 - c1)
void circumcentres_and_signs(Oracle &o) {
  const imodel_swm_mesh &m = o.m;
  const size_t ne = m.ne, nt = m.nt;
  if (!o.sgtg.empty()) return;
  std::vector<double> &cc = o.cc;
  cc.assign(3 * nt, 0.0);
  for (size_t k = 0; k < nt; ++k) {
    const double *p0 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k] - 1);
    const double *p1 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k + 1] - 1);
    const double *p2 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k + 2] - 1);
    double a[3], b[3], x[3];
    for (int i = 0; i < 3; ++i) {
      a[i] = p1[i] - p0[i];
      b[i] = p2[i] - p0[i];
    }
    x[0] = a[1] * b[2] - a[2] * b[1];
    x[1] = a[2] * b[0] - a[0] * b[2];
    x[2] = a[0] * b[1] - a[1] * b[0];
    const double side = x[0] * (p0[0] + p1[0] + p2[0]) + x[1] * (p0[1] + p1[1] + p2[1]) +
                        x[2] * (p0[2] + p1[2] + p2[2]);
    const double n = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) * (side < 0 ? -1.0 : 1.0);
    for (int i = 0; i < 3; ++i) cc[3 * k + i] = x[i] / n;
  }
  o.sgtg.assign(ne, 0.0);
  for (size_t l = 0; l < ne; ++l) {
    const double *c1 = &cc[3 * static_cast<size_t>(m.ed_sh[2 * l] - 1)];
    const double *c2 = &cc[3 * static_cast<size_t>(m.ed_sh[2 * l + 1] - 1)];
    const double *nr = m.ed_nr + 3 * l;
    const double d = nr[0] * (c2[0] - c1[0]) + nr[1] * (c2[1] - c1[1]) + nr[2] * (c2[2] - c1[2]);
    o.sgtg[l] = std::copysign(1.0, d);
  }
}

// coefficients as swm.f90:169-205 sets them: kf2 / kf4 (the "align" /
// "diam" fields, [nv]) or, where NULL, the constants k2 / k4 ("const"); the
// sign of grad_ed_tg from the triangles' circumcentres (trcircumc: the unit
// normal of the vertices' plane, on their side)
static int set_diffusion(Oracle &o, double k2, double k4, const double *kf2, const double *kf4) {
  const imodel_swm_mesh &m = o.m;
  if (!(k2 >= 0) || !(k4 >= 0)) return IMODEL_SWM_EINVAL;
  o.k2_on = k2 > 0 || kf2;
  o.k4_on = k4 > 0 || kf4;
  if (!o.k2_on && !o.k4_on) return IMODEL_SWM_OK;
  if (!m.ed_nr || !m.v_p) return IMODEL_SWM_EINVAL;
  const size_t nv = m.nv, ne = m.ne, nt = m.nt;
  const double *kf = o.k4_on ? kf4 : kf2;
  o.dif_hx.assign(nv, o.k4_on ? k4 : k2);
  if (kf) o.dif_hx.assign(kf, kf + nv);
  // scalar_hx2tr of the coefficient (:258-263)
  o.dif_tr.assign(nt, 0.0);
  for (size_t k = 0; k < nt; ++k) {
    double f = 0.0;
    for (int i = 0; i < 3; ++i) f = f + m.tr_trhx_area[3 * k + i] * o.dif_hx[m.tr_v[3 * k + i] - 1];
    o.dif_tr[k] = f / m.tr_areag[k];
  }
  if (o.k4_on) {
    for (size_t i = 0; i < nv; ++i) o.dif_hx[i] = std::sqrt(o.dif_hx[i]);
    for (size_t k = 0; k < nt; ++k) o.dif_tr[k] = std::sqrt(o.dif_tr[k]);
  }
  circumcentres_and_signs(o);
  for (auto *v : {&o.lapu, &o.lap_lapu}) v->assign(ne, 0.0);
  for (auto *v : {&o.coefvort, &o.vort_lap}) v->assign(nt, 0.0);
  for (auto *v : {&o.coefdiv, &o.div_lap}) v->assign(nv, 0.0);
  return IMODEL_SWM_OK;
}

int oracle_set_diffusion(void *p, double k2, double k4) {
  return set_diffusion(*static_cast<Oracle *>(p), k2, k4, nullptr, nullptr);
}

int oracle_set_diffusion_fields(void *p, const double *k2_hx, const double *k4_hx) {
  Oracle &o = *static_cast<Oracle *>(p);
  for (const double *f : {k2_hx, k4_hx})
    if (f)
      for (int i = 0; i < o.m.nv; ++i)
        if (!(f[i] >= 0) || !std::isfinite(f[i])) return IMODEL_SWM_EINVAL;
  return set_diffusion(o, 0.0, 0.0, k2_hx, k4_hx);
}

// vort_tr's Coriolis parameter (swm_operators.f90:592-601): fsphere 0
// 2.*Omega*dsin(lat), fsphere 2 the constant fcte
int oracle_set_fcor(void *p, int32_t fsphere, double fcte) {
  Oracle &o = *static_cast<Oracle *>(p);
  if (fsphere != 0 && fsphere != 2) return IMODEL_SWM_EINVAL;
  for (int k = 0; k < o.m.nt; ++k)
    o.fcor[k] = fsphere == 2 ? fcte : 2.0 * o.m.omega * std::sin(o.m.tr_c_lat[k]);
  return IMODEL_SWM_OK;
}

int oracle_set_apvm(void *p, double pvspar, double dt) {
  Oracle &o = *static_cast<Oracle *>(p);
  const imodel_swm_mesh &m = o.m;
  if (!(pvspar >= 0) || !std::isfinite(pvspar)) return IMODEL_SWM_EINVAL;
  o.apvm_on = pvspar > 0;
  if (!o.apvm_on) return IMODEL_SWM_OK;
  if (!(dt > 0) || !std::isfinite(dt) || !m.ed_nr || !m.ed_c || !m.v_p) {
    o.apvm_on = false;
    return IMODEL_SWM_EINVAL;
  }
  o.pvspar = pvspar;
  o.apvm_dt = dt;
  circumcentres_and_signs(o);
  o.q_grad_ed.assign(m.ne, 0.0);
  o.q_grad_tr.assign(3 * static_cast<size_t>(m.nt), 0.0);
  return IMODEL_SWM_OK;
}

// the method wrapper of swm.par (swm_data.f90:446-507) and the geometry its
// branches read, as initialize_gridprop precomputes it (swm.f90:1005-1028):
// tr%c%b = bar_coord_tr(tr%c%p) (smeshpack.f90:5200-5245) for pxt16, the
// circumcentre distances of scalar_tr2ed's bary branch and of dtred, the
// kite-free edge areas of scalar_edtr2trcc and the edge connections of the
// gass Coriolis term
int oracle_set_scheme(void *p, int32_t scheme) {
  Oracle &o = *static_cast<Oracle *>(p);
  const imodel_swm_mesh &m = o.m;
  if (scheme < 0 || scheme > 3) return IMODEL_SWM_EINVAL;
  if (scheme != 0 && (!m.ed_nr || !m.ed_c || !m.v_p)) return IMODEL_SWM_EINVAL;
  o.scheme = scheme;
  if (scheme == 0) return IMODEL_SWM_OK;
  const size_t nv = m.nv, ne = m.ne, nt = m.nt;
  (void)nv;
  circumcentres_and_signs(o);
  o.h_trk.assign(nt, 0.0);
  if (scheme == 1) {
    o.bary.assign(3 * nt, 0.0);
    for (size_t k = 0; k < nt; ++k) {
      const double *pc = &o.cc[3 * k];
      const double *p1 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k] - 1);
      const double *p2 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k + 1] - 1);
      const double *p3 = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * k + 2] - 1);
      double b[3] = {std::fabs(det3(pc, p2, p3)), std::fabs(det3(pc, p3, p1)),
                     std::fabs(det3(pc, p1, p2))};
      double area = b[0];
      area = area + b[1];
      area = area + b[2];
      for (int i = 0; i < 3; ++i) o.bary[3 * k + i] = b[i] / area;
    }
  }
  if (scheme == 1 || scheme == 3) {
    o.dist.assign(2 * ne, 0.0);
    for (size_t l = 0; l < ne; ++l)
      for (int i = 0; i < 2; ++i)
        o.dist[2 * l + i] =
            arclen(m.ed_c + 3 * l, &o.cc[3 * static_cast<size_t>(m.ed_sh[2 * l + i] - 1)]);
  }
  if (scheme == 2) {
    o.edarea.assign(3 * nt, 0.0);
    for (size_t k = 0; k < nt; ++k)
      for (int i = 0; i < 3; ++i) {
        const int ed = m.tr_ed[3 * k + i] - 1;
        o.edarea[3 * k + i] =
            sphtriarea(&o.cc[3 * k], m.v_p + 3 * static_cast<size_t>(m.ed_v[2 * ed] - 1),
                       m.v_p + 3 * static_cast<size_t>(m.ed_v[2 * ed + 1] - 1));
      }
    o.h_rhb.assign(ne, 0.0);
    o.conn.assign(12 * ne, -2);
    for (size_t l = 0; l < ne; ++l)
      for (int i = 0; i < 2; ++i) {
        const int node = m.ed_v[2 * l + i] - 1;
        for (int j = 0; j < m.nnb[node]; ++j)
          o.conn[12 * l + 6 * i + j] =
              edge_connection(m, static_cast<int>(l), m.v_ed[I6(node, j)] - 1);
      }
  }
  if (scheme == 3) o.vhq_tr.assign(3 * nt, 0.0);
  return IMODEL_SWM_OK;
}

int oracle_tendency(void *p, const double *h, const double *u, double *masseq, double *momeq) {
  return tendency(*static_cast<Oracle *>(p), h, u, masseq, momeq);
}

int oracle_rk4(void *p, const double *h, const double *u, double *h_new, double *u_new,
               double dt) {
  return rk4(*static_cast<Oracle *>(p), h, u, h_new, u_new, dt);
}

// time loop of swm_tests (swm.f90:238-370) without diagnostics or output:
// ode_rk4(h_old, u_old -> h, u); u_old = u; h_old = h
int oracle_run(void *p, double *h, double *u, double dt, int32_t nsteps) {
  Oracle &o = *static_cast<Oracle *>(p);
  for (int k = 0; k < nsteps; ++k) {
    int rc = rk4(o, h, u, o.h_tmp.data(), o.u_tmp.data(), dt);
    if (rc) return rc;
    std::memcpy(h, o.h_tmp.data(), sizeof(double) * o.m.nv);
    std::memcpy(u, o.u_tmp.data(), sizeof(double) * o.m.ne);
  }
  return IMODEL_SWM_OK;
}

// calc_energies (swm.f90:2686-2752) + sumf_areas + RMS divergence; h_ed and
// divu are those of the last tendency evaluation, as in the reference.
int oracle_diagnostics(void *p, const double *h, const double *u, imodel_swm_diag *out) {
  Oracle &o = *static_cast<Oracle *>(p);
  const imodel_swm_mesh &m = o.m;
  const double grav = m.grav;
  std::memset(out, 0, sizeof(*out));
  out->mass = sumf_areas_cells(m, h);
  double pe = 0.0;
  for (int i = 0; i < m.nv; ++i) pe = pe + m.hx_areag[i] * grav * h[i] * (h[i] * 0.5 + o.bt[i]);
  std::vector<double> hbt(m.nv);
  for (int i = 0; i < m.nv; ++i) hbt[i] = h[i] + o.bt[i];
  double mean_height = sumf_areas_cells(m, hbt.data());
  double unavail = 0.0;
  for (int i = 0; i < m.nv; ++i) {
    double mhb = mean_height - o.bt[i];
    unavail = unavail + m.hx_areag[i] * grav * mhb * (mhb * 0.5 + o.bt[i]);
  }
  double ke = 0.0;
  for (int l = 0; l < m.ne; ++l)
    ke = ke + 0.5 * m.ed_leng[l] * m.edhx_leng[l] * o.h_ed[l] * (u[l] * u[l]);
  out->penergy = pe;
  out->kenergy = ke;
  out->tenergy = pe + ke;
  out->availenergy = out->tenergy - unavail;
  // potential enstrophy with the kite-weighted depth at the triangles, whatever
  // the scheme's own h_tr
  double ens = 0.0;
  if (o.scheme == 0 || o.scheme == 3) {
    for (int k = 0; k < m.nt; ++k) ens = ens + m.tr_areag[k] * o.h_tr[k] * (o.q_tr[k] * o.q_tr[k]) * 0.5;
  } else {
    for (int k = 0; k < m.nt; ++k) {
      const double ht = o.h_trk[k];
      const double q = ht != 0.0 ? o.eta[k] / ht : 0.0;
      ens = ens + m.tr_areag[k] * ht * (q * q) * 0.5;
    }
  }
  out->pot_enstrophy = ens;
  out->rms_div = std::sqrt(sumfsq_areas(m, o.divu.data(), 0));
  double mx = 0.0;
  for (int i = 0; i < m.nv; ++i) mx = std::fmax(mx, std::fabs(o.divu[i]));
  out->max_div = mx;
  int bad = 0;
  for (int i = 0; i < m.nv; ++i) bad |= !std::isfinite(h[i]);
  for (int l = 0; l < m.ne; ++l) bad |= !std::isfinite(u[l]);
  out->nan_found = bad;
  return IMODEL_SWM_OK;
}

// error_calc, swm.f90:3492-3543: out = {errormaxrel, error2rel, errormax}
int oracle_error_calc(void *p, const double *f, const double *fref, int32_t pos, double out[3]) {
  Oracle &o = *static_cast<Oracle *>(p);
  const imodel_swm_mesh &m = o.m;
  int n = pos == 0 ? m.nv : (pos == 1 ? m.nt : m.ne);
  std::vector<double> dif(n);
  for (int i = 0; i < n; ++i) dif[i] = f[i] - fref[i];
  double refsum = sumfsq_areas(m, fref, pos);
  double e2 = refsum > 0 ? std::sqrt(sumfsq_areas(m, dif.data(), pos)) / std::sqrt(refsum)
                         : std::sqrt(sumfsq_areas(m, dif.data(), pos));
  double refmax = 0.0, emax = 0.0;
  for (int i = 0; i < n; ++i) {
    refmax = std::fmax(refmax, std::fabs(fref[i]));
    emax = std::fmax(emax, std::fabs(dif[i]));
  }
  out[0] = refmax > 0 ? emax / refmax : emax;
  out[1] = e2;
  out[2] = emax;
  return IMODEL_SWM_OK;
}

// vecrecon_trsk_tg, interpack.f90:3852-3976 (var%pos == 6), scalar utg
int oracle_trsk_tangent(void *p, const double *u, double *utg) {
  Oracle &o = *static_cast<Oracle *>(p);
  const imodel_swm_mesh &m = o.m;
  int nth = o.nthreads;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nth) reduction(+ : bad)
  for (int ed = 0; ed < m.ne; ++ed) {
    double t = 0.0;
    for (int i = 0; i < 2; ++i) {
      int cell = m.ed_v[2 * ed + i] - 1;
      int ed_celli = getedindexonhx(m, ed, cell);
      if (ed_celli == 0) {
        bad += 1;
        continue;
      }
      for (int j = 0; j < m.nnb[cell]; ++j) {
        int k = m.v_ed[I6(cell, j)] - 1;
        double signcor =
            -1.0 * m.hx_ttgout[I6(cell, j)] * m.hx_tnrccw[I6(cell, ed_celli - 1)];
        double w = m.hx_trskw[static_cast<size_t>(cell) * 36 + static_cast<size_t>(j) * 6 +
                              (ed_celli - 1)];
        t = t + u[k] * m.edhx_leng[k] * w * signcor;
      }
    }
    utg[ed] = t / m.ed_leng[ed];
  }
  return bad ? IMODEL_SWM_EINVAL : IMODEL_SWM_OK;
}

// calc_trisk_weights, interpack.f90:4046-4095, from hx%hxtr_area
int oracle_trsk_weights(const imodel_swm_mesh *m, double *trskw) {
  for (int c = 0; c < m->nv; ++c) {
    int n = m->nnb[c];
    const double *R = m->hx_hxtr_area + I6(c, 0);
    for (int q = 0; q < 36; ++q) trskw[static_cast<size_t>(c) * 36 + q] = 0.0;
    for (int i = 1; i <= n; ++i) {
      for (int j = 1; j <= n; ++j) {
        double rsum = 0.0;
        double w;
        if (i == j) {
          w = 0.0;
        } else {
          if (j < i) {
            for (int k = i; k <= n; ++k) rsum = rsum + R[k - 1];
            for (int k = 1; k <= j - 1; ++k) rsum = rsum + R[k - 1];
          } else {
            for (int k = i; k <= j - 1; ++k) rsum = rsum + R[k - 1];
          }
          w = rsum - 0.5;
        }
        trskw[static_cast<size_t>(c) * 36 + static_cast<size_t>(j - 1) * 6 + (i - 1)] = w;
      }
    }
  }
  return IMODEL_SWM_OK;
}

// initialize_fields, testcase 2 with HTC staggering (swm.f90:1205-1262)
int oracle_tc2(const imodel_swm_mesh *m, double *h, double *u) {
  const double erad = m->erad, omega = m->omega;
  const double gravi = 1.0 / m->grav;
  const double pi2 = 2.0 * kPi;
  const double day2sec = 86400.0;
  const double u0 = pi2 * erad / (12.0 * day2sec);
  const double h0 = 2.94e4 * gravi;
  const double h_ct = (erad * omega * u0 + (u0 * u0) / 2.0) * gravi;
  for (int i = 0; i < m->nv; ++i) {
    double s = std::sin(m->v_lat[i]);
    h[i] = h0 - h_ct * (s * s);
  }
  for (int l = 0; l < m->ne; ++l) {
    const double *p = m->ed_c + 3 * static_cast<size_t>(l);
    const double *tg = m->ed_tg + 3 * static_cast<size_t>(l);
    double utmp = u0 * std::cos(m->ed_c_lat[l]);
    double vtmp = 0.0;
    // convert_vec_sph2cart, smeshpack.f90:4379-4417
    double rho = std::sqrt(p[0] * p[0] + p[1] * p[1]);
    double v[3];
    if (rho == 0.0) {
      v[0] = vtmp;
      v[1] = utmp;
      v[2] = 0.0;
    } else {
      v[0] = -(utmp * (p[1] / rho)) - (vtmp * p[0] * p[2]) / rho;
      v[1] = utmp * (p[0] / rho) - (vtmp * p[1] * p[2]) / rho;
      v[2] = vtmp * rho;
    }
    double d = v[0] * tg[0];
    d = d + v[1] * tg[1];
    d = d + v[2] * tg[2];
    u[l] = d;
  }
  return IMODEL_SWM_OK;
}

int oracle_field(void *p, int32_t which, double *out) {
  Oracle &o = *static_cast<Oracle *>(p);
  const std::vector<double> *v = nullptr;
  switch (which) {
    case 0: v = &o.h_ed; break;
    case 1: v = &o.uh; break;
    case 2: v = &o.eta; break;
    case 3: v = &o.h_tr; break;
    case 4: v = &o.q_tr; break;
    case 5: v = &o.q_ed; break;
    case 6: v = &o.divuh; break;
    case 7: v = &o.ke; break;
    case 8: v = &o.ghbK; break;
    case 9: v = &o.grad; break;
    case 10: v = &o.uhq; break;
    case 11: v = &o.divu; break;
    case 12: v = &o.zeta; break;
    case 13: v = &o.eta_ed; break;
    case 14: v = &o.lapu; break;       // with diffusion on
    case 15: v = &o.lap_lapu; break;   // with hyperdiffusion on
    case 16: v = &o.q_grad_ed; break;  // with apvm on
    case 17: v = &o.h_rhb; break;      // gass18
    case 18: v = &o.vhq_tr; break;     // dtred [nt][3]
    case 19: v = &o.vhx; break;        // Perot velocity at the cells [nv][3]
    default: return IMODEL_SWM_EINVAL;
  }
  if (v->empty()) return IMODEL_SWM_ESTATE;
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return IMODEL_SWM_OK;
}

}  // extern "C"

// ---- the moist shallow-water model (moist_swm.f90) ------------------------
// Tracers h theta, h qv, h qc, h qr and a passive h tracer advected with
// advmtd = "trsk" (divhx, highorder.f90:4901-4983: div_hx of u times
// scalar_hx2ed of the tracer), the thermal momentum source and the
// condensation / precipitation sources (source, moist_swm.f90:1278-1353),
// classic RK4 (ode_rk4_moist_swm, :1819-2011, no monotonic filter).  theta,
// qv, qc, qr are the module fields the sources read: theta keeps its
// initial value in the RK4 path (nothing updates it there), qv, qc, qr are
// hqv / h etc. after each step (moist_swm_tests, :1531-1533).
struct MoistOracle {
  Oracle *base;
  int testcase;
  int upw1 = 0;  // advmtd: 0 = "trsk", 1 = "upw1"
  double q0, dt;
  std::vector<double> theta, qv, qc, qr;
  std::vector<double> f[7][4];          // tendencies of the 7 fields per stage
  std::vector<double> stage_in[7], tmp_out[7];
  std::vector<double> uphi, div, su, hs[4];
};

namespace {
constexpr double kLscale = 10.0, kGammaR = 0.001, kQprecip = 0.0001;

// tendency_advection (highorder.f90:3936-3972) with advmtd = "trsk"
// (divhx, :4967-4974: scalar_hx2ed, scalar_elem_product, div_hx) or "upw1"
// (div_hx_upw1, :5094-5139: the first-order upwind flux, the cell's own
// value where the flux leaves it, the neighbour's where it enters)
void advection(MoistOracle &mo, const double *q, const double *u, double *phif) {
  const imodel_swm_mesh &m = mo.base->m;
  const int nv = m.nv, ne = m.ne, nth = mo.base->nthreads;
  if (mo.upw1) {
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int i = 0; i < nv; ++i) {
      double d = 0.0;
      for (int j = 0; j < m.nnb[i]; ++j) {
        const int l = m.v_ed[I6(i, j)] - 1;
        const int k = m.v_nb[I6(i, j)] - 1;
        const double signcor = static_cast<double>(m.hx_ttgout[I6(i, j)]);
        if (signcor * u[l] > 0.0)
          d = d + signcor * u[l] * m.edhx_leng[l] * q[i];
        else
          d = d + signcor * u[l] * m.edhx_leng[l] * q[k];
      }
      d = d / m.hx_areag[i] / m.erad;
      phif[i] = -d;
    }
    return;
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int l = 0; l < ne; ++l) {
    const double qe = (q[m.ed_v[2 * l] - 1] + q[m.ed_v[2 * l + 1] - 1]) * 0.5;
    mo.uphi[l] = u[l] * qe;
  }
#pragma omp parallel for schedule(static) num_threads(nth)
  for (int i = 0; i < nv; ++i) {
    double d = 0.0;
    for (int j = 0; j < m.nnb[i]; ++j) {
      const int l = m.v_ed[I6(i, j)] - 1;
      const double signcor = static_cast<double>(m.hx_ttgout[I6(i, j)]);
      d = d + signcor * mo.uphi[l] * m.edhx_leng[l];
    }
    phif[i] = -(d / m.hx_areag[i] / m.erad);
  }
}

// qsat (moist_swm.f90:618-622)
inline double qsat(double T, double H, double B, double q0, double grav) {
  return q0 * std::exp(20.0 * T) / ((H + B) * grav);
}

// tendency_moist_swm (moist_swm.f90:1151-1276) for RK4; out[0..6] = masseq,
// momeq, tempeq, vapoureq, cloudeq, raineq, tracereq
int moist_tendency(MoistOracle &mo, const double *const in[7], double *const out[7]) {
  Oracle &o = *mo.base;
  const imodel_swm_mesh &m = o.m;
  const int nv = m.nv, ne = m.ne, nth = o.nthreads;
  const double grav = m.grav, gravo2 = grav * 0.5, erad = m.erad;
  const double *h = in[0], *u = in[1];
  if (mo.testcase > 1) {
    int rc = tendency(o, h, u, out[0], out[1]);
    if (rc) return rc;
    for (int k = 2; k < 6; ++k) advection(mo, in[k], u, out[k]);
    if (mo.testcase == 2) advection(mo, in[6], u, out[6]);
    // source (moist_swm.f90:1278-1353): momentum, from h^2 theta and the
    // topography; h_ed is the tendency's
    int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nth) reduction(+ : bad)
    for (int l = 0; l < ne; ++l) {
      const int v1 = m.ed_v[2 * l] - 1, v2 = m.ed_v[2 * l + 1] - 1;
      double g = h[v2] * in[2][v2] - h[v1] * in[2][v1];
      g = g / m.ed_leng[l] / erad;
      double gpi_oh = 0.0;
      if (std::fabs(o.h_ed[l]) < kEps / 100000.0)
        bad += 1;
      else
        gpi_oh = g / o.h_ed[l];
      double gb = o.bt[v2] - o.bt[v1];
      gb = gb / m.ed_leng[l] / erad;
      const double th_ed = (mo.theta[v1] + mo.theta[v2]) * 0.5;
      mo.su[l] = gravo2 * gpi_oh + grav * (th_ed * gb);
    }
    if (bad) return IMODEL_SWM_EDIVZERO;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int i = 0; i < nv; ++i) {
      const double qs = qsat(mo.theta[i], h[i], o.bt[i], mo.q0, grav);
      double gamma_v = 1.0 + kLscale * (20.0 * qs);
      gamma_v = 1.0 / gamma_v;
      double dqv = gamma_v * (mo.qv[i] - qs);
      dqv = std::max(0.0, dqv) / mo.dt;
      double dqc = std::max(0.0, -gamma_v * (mo.qv[i] - qs));
      dqc = std::min(mo.qc[i], dqc) / mo.dt;
      const double dqr = std::max(0.0, kGammaR * (mo.qc[i] - kQprecip)) / mo.dt;
      mo.hs[1][i] = h[i] * (dqc - dqv);
      mo.hs[2][i] = h[i] * (dqv - dqc - dqr);
      mo.hs[3][i] = h[i] * dqr;
      mo.hs[0][i] = h[i] * (kLscale * (dqv - dqc));
    }
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int l = 0; l < ne; ++l) out[1][l] = out[1][l] + mo.su[l];
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int i = 0; i < nv; ++i)
      for (int k = 0; k < 4; ++k) out[2 + k][i] = out[2 + k][i] + mo.hs[k][i];
  } else if (mo.testcase == 1) {
    advection(mo, in[6], u, out[6]);
  }
  return IMODEL_SWM_OK;
}
}  // namespace

extern "C" {

int oracle_moist_set_advection(void *h, int32_t upw1) {
  if (!h || (upw1 != 0 && upw1 != 1)) return 1;
  static_cast<MoistOracle *>(h)->upw1 = upw1;
  return 0;
}

void *oracle_moist_create(const imodel_swm_mesh *m, int32_t testcase, const double *bt,
                          const double *theta, double q0, int32_t nthreads) {
  if (!m || !theta || testcase < 1 || testcase > 5) return nullptr;
  MoistOracle *mo = new MoistOracle();
  mo->base = static_cast<Oracle *>(oracle_create(m, testcase, bt, nthreads));
  mo->testcase = testcase;
  mo->q0 = q0;
  const size_t nv = m->nv, ne = m->ne;
  mo->theta.assign(theta, theta + nv);
  mo->qv.assign(nv, 0.0);
  mo->qc.assign(nv, 0.0);
  mo->qr.assign(nv, 0.0);
  for (int k = 0; k < 7; ++k) {
    const size_t n = k == 1 ? ne : nv;
    for (int s = 0; s < 4; ++s) mo->f[k][s].assign(n, 0.0);
    mo->stage_in[k].assign(n, 0.0);
    mo->tmp_out[k].assign(n, 0.0);
  }
  mo->uphi.assign(ne, 0.0);
  mo->su.assign(ne, 0.0);
  for (int k = 0; k < 4; ++k) mo->hs[k].assign(nv, 0.0);
  return mo;
}

void oracle_moist_destroy(void *p) {
  MoistOracle *mo = static_cast<MoistOracle *>(p);
  if (!mo) return;
  oracle_destroy(mo->base);
  delete mo;
}

// the module fields qv, qc, qr the next step's sources read
int oracle_moist_set_q(void *p, const double *qv, const double *qc, const double *qr) {
  MoistOracle &mo = *static_cast<MoistOracle *>(p);
  const int nv = mo.base->m.nv;
  mo.qv.assign(qv, qv + nv);
  mo.qc.assign(qc, qc + nv);
  mo.qr.assign(qr, qr + nv);
  return IMODEL_SWM_OK;
}

// nsteps of the moist_swm_tests time loop: ode_rk4_moist_swm, then qv, qc,
// qr = hq / h (scalar_elem_divide with its guard).  y[7] = h, u, h theta,
// h qv, h qc, h qr, h tracer, advanced in place
int oracle_moist_run(void *p, double *const y[7], double dt, int32_t nsteps) {
  MoistOracle &mo = *static_cast<MoistOracle *>(p);
  const imodel_swm_mesh &m = mo.base->m;
  const int nv = m.nv, nth = mo.base->nthreads;
  mo.dt = dt;
  const size_t n[7] = {static_cast<size_t>(nv), static_cast<size_t>(m.ne), static_cast<size_t>(nv),
                       static_cast<size_t>(nv), static_cast<size_t>(nv), static_cast<size_t>(nv),
                       static_cast<size_t>(nv)};
  // which fields a stage advances: all for testcase > 1 (the tracer for
  // testcase 2 only), the tracer alone for testcase 1
  bool adv[7];
  for (int k = 0; k < 7; ++k)
    adv[k] = mo.testcase > 1 ? (k < 6 || mo.testcase == 2) : k == 6;
  for (int step = 0; step < nsteps; ++step) {
    const double *in[7];
    double *out[7];
    for (int k = 0; k < 7; ++k) in[k] = y[k];
    const double frac[3] = {0.5, 0.5, 1.0};
    for (int s = 0; s < 4; ++s) {
      for (int k = 0; k < 7; ++k) out[k] = mo.f[k][s].data();
      int rc = moist_tendency(mo, in, out);
      if (rc) return rc;
      if (s == 3) break;
      for (int k = 0; k < 7; ++k) {
        std::vector<double> &nx = mo.stage_in[k];
        const double *f0 = mo.f[k][s].data();
        const double *yk = y[k];
        if (!adv[k]) {
          std::memcpy(nx.data(), yk, n[k] * sizeof(double));
        } else if (frac[s] == 0.5) {
#pragma omp parallel for schedule(static) num_threads(nth)
          for (size_t i = 0; i < n[k]; ++i) nx[i] = yk[i] + dt * f0[i] / 2.0;
        } else {
#pragma omp parallel for schedule(static) num_threads(nth)
          for (size_t i = 0; i < n[k]; ++i) nx[i] = yk[i] + dt * f0[i];
        }
        in[k] = nx.data();
      }
    }
    for (int k = 0; k < 7; ++k) {
      if (!adv[k]) continue;
      const double *a = mo.f[k][0].data(), *b = mo.f[k][1].data(), *c = mo.f[k][2].data(),
                   *d = mo.f[k][3].data();
      double *yk = y[k];
#pragma omp parallel for schedule(static) num_threads(nth)
      for (size_t i = 0; i < n[k]; ++i)
        yk[i] = yk[i] + dt * (a[i] + 2.0 * b[i] + 2.0 * c[i] + d[i]) / 6.0;
    }
    int bad = 0;
    for (int i = 0; i < nv; ++i) {
      const double hi = y[0][i];
      if (std::fabs(hi) < kEps / 100000.0) {
        bad += 1;
        continue;
      }
      mo.qv[i] = y[3][i] / hi;
      mo.qc[i] = y[4][i] / hi;
      mo.qr[i] = y[5][i] / hi;
    }
    if (bad) return IMODEL_SWM_EDIVZERO;
  }
  return IMODEL_SWM_OK;
}

}  // extern "C"
