// Host construction of the device layout (see swm_layout.h).
#include "swm_layout.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace imodel {
namespace {

// 3-D Hilbert index of integer coordinates (b bits each), following the
// transpose formulation published by J. Skilling, "Programming the Hilbert
// curve", AIP Conf. Proc. 707 (2004).
uint64_t hilbert3(uint32_t x0, uint32_t x1, uint32_t x2, int b) {
  uint32_t X[3] = {x0, x1, x2};
  const uint32_t M = 1u << (b - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t key = 0;
  for (int bit = b - 1; bit >= 0; --bit)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> bit) & 1u);
  return key;
}

uint32_t quant(double x, int b) {
  const double s = static_cast<double>((1u << b) - 1);
  double q = (x + 1.0) * 0.5 * s + 0.5;
  if (q < 0) q = 0;
  if (q > s) q = s;
  return static_cast<uint32_t>(q);
}

// n2o: the indices 0..n-1 in the order of their keys, equal keys in index
// order (the order std::stable_sort gives), by a least-significant-digit
// radix sort of (key, index) pairs, 8-bit digits, skipping the digits that
// are the same in every key; o2n its inverse.  Each pass runs on host
// threads: every thread counts the digits of its own contiguous chunk, a
// prefix over (digit, thread) gives each thread its output positions, and
// each thread moves its chunk in order, so the pass stays stable.
template <class Key, class V>
void sort_perm(V &n2o, V &o2n, const std::vector<Key> &key) {
  const int64_t n = static_cast<int64_t>(key.size());
  HVec<Key> ka(key.begin(), key.end()), kb(key.size());
  V ia(key.size()), ib(key.size());
  Key any = 0, all = static_cast<Key>(~Key(0));
#pragma omp parallel for schedule(static) reduction(| : any) reduction(& : all)
  for (int64_t i = 0; i < n; ++i) {
    ia[i] = static_cast<int32_t>(i);
    any |= key[i];
    all &= key[i];
  }
#ifdef _OPENMP
  const int tmax = omp_get_max_threads();
#else
  const int tmax = 1;
#endif
  std::vector<int64_t> cnt(static_cast<size_t>(tmax) * 256);
  for (int shift = 0; shift < static_cast<int>(8 * sizeof(Key)); shift += 8) {
    if ((((any ^ all) >> shift) & 0xFF) == 0) continue;
#pragma omp parallel num_threads(tmax)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num(), nth = omp_get_num_threads();
#else
      const int t = 0, nth = 1;
#endif
      const int64_t lo = n * t / nth, hi = n * (t + 1) / nth;
      int64_t *c = &cnt[static_cast<size_t>(t) * 256];
      for (int d = 0; d < 256; ++d) c[d] = 0;
      for (int64_t i = lo; i < hi; ++i) ++c[(ka[i] >> shift) & 0xFF];
#pragma omp barrier
#pragma omp single
      {
        int64_t acc = 0;
        for (int d = 0; d < 256; ++d)
          for (int u = 0; u < nth; ++u) {
            const int64_t v = cnt[static_cast<size_t>(u) * 256 + d];
            cnt[static_cast<size_t>(u) * 256 + d] = acc;
            acc += v;
          }
      }
      for (int64_t i = lo; i < hi; ++i) {
        const int64_t to = c[(ka[i] >> shift) & 0xFF]++;
        kb[to] = ka[i];
        ib[to] = ia[i];
      }
    }
    ka.swap(kb);
    ia.swap(ib);
  }
  n2o.swap(ia);
  o2n.resize(key.size());
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) o2n[n2o[i]] = static_cast<int32_t>(i);
}

// body(i) for i in [0, n) on host threads; body returns "" or an error
// message, and the message of the lowest failing i comes back: the one a
// serial loop would have stopped at
template <class F>
std::string par_for(int64_t n, F body) {
  int64_t first = INT64_MAX;
  std::string msg;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    std::string e = body(i);
    if (!e.empty()) {
#pragma omp critical(imodel_layout_first_error)
      if (i < first) {
        first = i;
        msg = std::move(e);
      }
    }
  }
  return msg;
}

// v = n copies of x, filled on host threads
template <class V, class T>
void fill(V &v, size_t n, T x) {
  v.resize(n);
  const int64_t m = static_cast<int64_t>(n);
  typename V::value_type *d = v.data();
  const typename V::value_type y = static_cast<typename V::value_type>(x);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) d[i] = y;
}

// tr%c%p of triangle t (0-based): the unit normal of the plane through its
// vertices, on their side of the origin -- the direction of the spherical
// circumcentre.  The oracle evaluates the same expressions.
void circumcentre(const imodel_swm_mesh &m, int t, double c[3]) {
  const double *p[3];
  for (int k = 0; k < 3; ++k)
    p[k] = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * static_cast<size_t>(t) + k] - 1);
  const double a[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
  const double b[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
  const double x[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                       a[0] * b[1] - a[1] * b[0]};
  const double side = x[0] * (p[0][0] + p[1][0] + p[2][0]) +
                      x[1] * (p[0][1] + p[1][1] + p[2][1]) + x[2] * (p[0][2] + p[1][2] + p[2][2]);
  const double nrm = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  for (int k = 0; k < 3; ++k) c[k] = (side < 0 ? -x[k] : x[k]) / nrm;
}

// spherical geometry as smeshpack.f90 evaluates it (no contraction: this
// file is compiled with -ffp-contract=off)
double dot3(const double *a, const double *b) {
  double s = a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}
// det(p1, p2, p3) = cross_product(p1, p2) . p3 (smeshpack.f90:6560-6595)
double det3(const double *p1, const double *p2, const double *p3) {
  const double c[3] = {p1[1] * p2[2] - p1[2] * p2[1], p1[2] * p2[0] - p1[0] * p2[2],
                       p1[0] * p2[1] - p1[1] * p2[0]};
  return dot3(c, p3);
}
// arclen (smeshpack.f90:4624-4657; pi from the default-real literal of
// constants.f90:31)
double arclen(const double *p, const double *q) {
  const double s[3] = {p[0] + q[0], p[1] + q[1], p[2] + q[2]};
  const double d = dot3(s, s);
  if (d == 0.0) return 4.0 * static_cast<double>(0.78539816339744830961566f);
  if (d >= 4.0) return 0.0;
  return 2.0 * std::atan(std::sqrt((4.0 - d) / d));
}
// sphtriarea, L'Huilier's theorem (smeshpack.f90:4710-4762; the degeneracy
// tolerance eps/100 with eps = epsilon(1.))
double sphtriarea(const double *p1, const double *p2, const double *p3) {
  const double tol = static_cast<double>(1.1920928955078125e-07f) / 100.0;
  auto dist = [](const double *a, const double *b) {
    const double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return std::sqrt(dot3(d, d));
  };
  if (dist(p1, p2) < tol || dist(p2, p3) < tol || dist(p1, p3) < tol) return 0.0;
  const double a = arclen(p1, p2), b = arclen(p2, p3), c = arclen(p3, p1);
  const double s = (a + b + c) / 2.0;
  double t = std::tan(s / 2.0) * std::tan((s - a) / 2.0);
  t = t * std::tan((s - b) / 2.0);
  t = t * std::tan((s - c) / 2.0);
  if (t < 0.0) return 0.0;
  return 4.0 * std::atan(std::sqrt(t));
}

// The edge whose PV the gass Coriolis term uses for stencil edge ed2 of edge
// ed1 (0-based, reference numbering): the third edge of a triangle holding
// both, else an edge joining a triangle of ed2's dual edge to a triangle
// holding ed1; -1 when ed1 == ed2 or they are further apart (the TRSK
// average is then used).  Restates getedgeintriangle and
// gethxedgeconnection, smeshpack.f90:4127-4244.
int edge_connection(const imodel_swm_mesh &m, int ed1, int ed2) {
  if (ed1 == ed2) return -1;
  auto tri_ed = [&](int t, int i) { return m.tr_ed[3 * static_cast<size_t>(t) + i] - 1; };
  auto tri_of = [&](int e, int s) { return m.ed_sh[2 * static_cast<size_t>(e) + s] - 1; };
  const int tr1 = tri_of(ed1, 0), tr2 = tri_of(ed1, 1);
  int tr = -1;
  for (int i = 0; i < 3 && tr < 0; ++i) {
    if (ed2 == tri_ed(tr1, i))
      tr = tr1;
    else if (ed2 == tri_ed(tr2, i))
      tr = tr2;
  }
  if (tr >= 0)
    for (int i = 0; i < 3; ++i)
      if (tri_ed(tr, i) != ed1 && tri_ed(tr, i) != ed2) return tri_ed(tr, i);
  for (int j = 0; j < 2; ++j) {
    const int trj = tri_of(ed2, j);
    for (int i = 0; i < 3; ++i) {
      const int edtmp = tri_ed(trj, i);
      if (edtmp == ed2) continue;
      const int a = tri_of(edtmp, 0);
      const int other = a == trj ? tri_of(edtmp, 1) : a;
      for (int k = 0; k < 3; ++k)
        if (ed1 == tri_ed(other, k)) return edtmp;
    }
  }
  return -1;
}

// The FP32 coefficients of the pxt16, gass18 and dtred branches (Layout:
// t_kite32, e_qw32, e_stc32, e_dtc32), from the FP64 geometry of the same
// branches, which build_layout has filled in device order before.
std::string scheme_fp32(const imodel_swm_mesh &m, Layout &L, int scheme) {
  const size_t NV = L.nv, NE = L.ne, NT = L.nt;
  (void)NV;
  const int ne = L.ne, nt = L.nt;
  if (scheme == IMODEL_SWM_PXT16 || scheme == IMODEL_SWM_GASS18) {
    // the depth at the triangle as weights of its vertices
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nt; ++i) {
      const int t = L.tri_n2o[i];
      double w[3] = {0.0, 0.0, 0.0};
      if (scheme == IMODEL_SWM_PXT16) {
        for (int s = 0; s < 3; ++s) w[s] = L.t_bary[s * NT + i];
      } else {
        // sum_s edarea_s (h_a + h_b) / 2 / A over the triangle's edges
        const double A = m.tr_areag[t];
        for (int s = 0; s < 3; ++s) {
          const int e = m.tr_ed[3 * static_cast<size_t>(t) + s] - 1;
          for (int end = 0; end < 2; ++end) {
            const int c = m.ed_v[2 * static_cast<size_t>(e) + end] - 1;
            for (int q = 0; q < 3; ++q)
              if (m.tr_v[3 * static_cast<size_t>(t) + q] - 1 == c)
                w[q] += 0.5 * L.t_edarea[s * NT + i] / A;
          }
        }
      }
      for (int s = 0; s < 3; ++s) L.t_kite32[s * NT + i] = static_cast<float>(w[s]);
    }
    // q_e from the edge's two triangles
    fill(L.e_qw32, 2 * NE, 0.0f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i) {
      double a, b;
      if (scheme == IMODEL_SWM_PXT16) {
        a = L.e_dist[NE + i];  // triangle 1 takes the other one's distance
        b = L.e_dist[i];
      } else {
        a = L.t_areag[L.e_sh[i]];
        b = L.t_areag[L.e_sh[NE + i]];
      }
      L.e_qw32[i] = static_cast<float>(a / (a + b));
      L.e_qw32[NE + i] = static_cast<float>(b / (a + b));
    }
  }
  if (scheme == IMODEL_SWM_PXT16) {
    // the q_e weights by cell slot, for the cell-centred variants: slot j's
    // edge lies between the cell's triangles j - 1 and j (c_tr);
    // c_qw32[2 j] weighs triangle j - 1, c_qw32[2 j + 1] triangle j
    const int nv = L.nv;
    fill(L.c_qw32, 12 * NV, 0.0f);
    const std::string err = par_for(nv, [&](int64_t i64) -> std::string {
      const int i = static_cast<int>(i64);
      const int n = L.c_nnb[i];
      for (int j = 0; j < n; ++j) {
        const int ie = L.c_ed[j * NV + i];
        const int ta = L.c_tr[((j + n - 1) % n) * NV + i], tb = L.c_tr[j * NV + i];
        const int t1 = L.e_sh[ie], t2 = L.e_sh[NE + ie];
        if (!((ta == t1 && tb == t2) || (ta == t2 && tb == t1)))
          return "cell " + std::to_string(L.cell_n2o[i] + 1) + ": slot " + std::to_string(j) +
                 "'s edge does not lie between the slot's triangles";
        L.c_qw32[static_cast<size_t>(2 * j) * NV + i] = ta == t1 ? L.e_qw32[ie] : L.e_qw32[NE + ie];
        L.c_qw32[static_cast<size_t>(2 * j + 1) * NV + i] = tb == t1 ? L.e_qw32[ie] : L.e_qw32[NE + ie];
      }
      return std::string();
    });
    if (!err.empty()) return err;
  }
  if (scheme == IMODEL_SWM_PXT16) {
    // pered on the TRSK stencil's slots, in the order build_layout made them
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i) {
      const int e = L.edge_n2o[i];
      const double *nr = m.ed_nr + 3 * static_cast<size_t>(e);
      int ns = 0;
      for (int s = 0; s < 2; ++s) {
        const int node = m.ed_v[2 * static_cast<size_t>(e) + s] - 1;
        const int n = m.nnb[node];
        int own = -1;
        for (int j = 0; j < n; ++j)
          if (m.v_ed[6 * static_cast<size_t>(node) + j] - 1 == e) own = j;
        for (int j = 0; j < n; ++j) {
          if (j == own) continue;
          const int k = m.v_ed[6 * static_cast<size_t>(node) + j] - 1;
          double d = 0.0;
          for (int c = 0; c < 3; ++c)
            d += (m.ed_c[3 * static_cast<size_t>(k) + c] - m.v_p[3 * static_cast<size_t>(node) + c]) *
                 nr[c];
          const double sg = static_cast<double>(m.hx_ttgout[6 * static_cast<size_t>(node) + j]);
          L.e_stc32[ns * NE + i] =
              static_cast<float>(-0.25 * sg * d * m.edhx_leng[k] / m.hx_areag[node]);
          ++ns;
        }
      }
    }
    // the same coefficients by cell, for the cell-centred variants
    const int nv = L.nv;
    fill(L.c_C32, 36 * NV, 0.0f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i) {
      const int c = L.cell_n2o[i];
      const int n = m.nnb[c];
      for (int si = 0; si < n; ++si) {
        const int e = m.v_ed[6 * static_cast<size_t>(c) + si] - 1;
        const double *nr = m.ed_nr + 3 * static_cast<size_t>(e);
        for (int j = 0; j < n; ++j) {
          if (j == si) continue;
          const int k = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
          double d = 0.0;
          for (int q = 0; q < 3; ++q)
            d += (m.ed_c[3 * static_cast<size_t>(k) + q] - m.v_p[3 * static_cast<size_t>(c) + q]) * nr[q];
          const double sg = static_cast<double>(m.hx_ttgout[6 * static_cast<size_t>(c) + j]);
          L.c_C32[static_cast<size_t>(6 * si + j) * NV + i] = static_cast<float>(
              -0.25 * sg * d * m.edhx_leng[k] / m.hx_areag[c] * m.ed_leng[e]);
        }
      }
    }
  }
  if (scheme == IMODEL_SWM_DTRED) {
    fill(L.e_dtc32, 6 * NE, 0.0f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i) {
      const double d1 = L.e_dist[i], d2 = L.e_dist[NE + i];
      const double w[2] = {d2 / (d1 + d2), d1 / (d1 + d2)};
      const double nr[3] = {L.e_nr[i], L.e_nr[NE + i], L.e_nr[2 * NE + i]};
      for (int si = 0; si < 2; ++si) {
        const int ti = L.e_sh[si * NE + i];
        const double tc[3] = {L.t_c[ti], L.t_c[NT + ti], L.t_c[2 * NT + ti]};
        for (int s = 0; s < 3; ++s) {
          const int ed = L.t_ed[s * NT + ti];
          const double ec[3] = {L.e_c[ed], L.e_c[NE + ed], L.e_c[2 * NE + ed]};
          const double cr[3] = {tc[1] * ec[2] - tc[2] * ec[1], tc[2] * ec[0] - tc[0] * ec[2],
                                tc[0] * ec[1] - tc[1] * ec[0]};
          const double dn = cr[0] * nr[0] + cr[1] * nr[1] + cr[2] * nr[2];
          const double sg = L.t_lt[s * NT + ti] < 0.0 ? -1.0 : 1.0;
          L.e_dtc32[(3 * si + s) * NE + i] =
              static_cast<float>(-w[si] * sg * L.e_leng[ed] * dn / L.t_areag[ti]);
        }
      }
    }
    // the same by triangle, for the cell-centred variants: the Perot
    // vector of uh at each triangle, P_t = sum_s uh_s a_ts with a_ts =
    // sign(tr%tg) l_s (tr%c x ed(s)%c) / tr%areag, the corner opposite each
    // edge slot (the edge's depth is the mean of the other two), and per
    // edge nr_e and the weights w_i
    fill(L.t_dpa32, 9 * NT, 0.0f);
    L.t_dopp.resize(NT);
    const std::string err = par_for(nt, [&](int64_t i64) -> std::string {
      const int ti = static_cast<int>(i64);
      const double tc[3] = {L.t_c[ti], L.t_c[NT + ti], L.t_c[2 * NT + ti]};
      uint8_t opp = 0;
      for (int s = 0; s < 3; ++s) {
        const int ed = L.t_ed[s * NT + ti];
        const double ec[3] = {L.e_c[ed], L.e_c[NE + ed], L.e_c[2 * NE + ed]};
        const double cr[3] = {tc[1] * ec[2] - tc[2] * ec[1], tc[2] * ec[0] - tc[0] * ec[2],
                              tc[0] * ec[1] - tc[1] * ec[0]};
        const double sg = L.t_lt[s * NT + ti] < 0.0 ? -1.0 : 1.0;
        for (int k = 0; k < 3; ++k)
          L.t_dpa32[(3 * s + k) * NT + ti] =
              static_cast<float>(sg * L.e_leng[ed] * cr[k] / L.t_areag[ti]);
        int o = -1;
        for (int q = 0; q < 3; ++q) {
          const int c = L.t_v[q * NT + ti];
          if (c != L.e_v[ed] && c != L.e_v[NE + ed]) o = q;
        }
        if (o < 0) return "triangle " + std::to_string(L.tri_n2o[ti] + 1) + ": edge slot " +
                          std::to_string(s) + " has no opposite corner";
        opp = static_cast<uint8_t>(opp | (o << (2 * s)));
      }
      L.t_dopp[ti] = opp;
      return std::string();
    });
    if (!err.empty()) return err;
    L.e_nr32.resize(3 * NE);
    L.e_dw32.resize(2 * NE);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i) {
      const double d1 = L.e_dist[i], d2 = L.e_dist[NE + i];
      L.e_dw32[i] = static_cast<float>(d2 / (d1 + d2));
      L.e_dw32[NE + i] = static_cast<float>(d1 / (d1 + d2));
      for (int k = 0; k < 3; ++k) L.e_nr32[k * NE + i] = static_cast<float>(L.e_nr[k * NE + i]);
    }
  }
  if (scheme == IMODEL_SWM_GASS18) {
    // the connecting edges by cell, for the cell-centred variants: on the
    // grid's hexagons and pentagons the connecting edge of two cell edges is
    // the outer edge of their triangle when they are adjacent, the edge
    // between them when one edge lies between, none when they are opposite;
    // gass_cells records that every cell follows that rule (the kernels
    // then need no per-pair table)
    const int nv = L.nv;
    L.c_gout.resize(6 * NV);
    const std::string err = par_for(nv, [&](int64_t i64) -> std::string {
      const int i = static_cast<int>(i64);
      const int c = L.cell_n2o[i];
      const int n = m.nnb[c];
      const std::string off = "cell " + std::to_string(c + 1);
      int outer[6];
      for (int t = 0; t < 6; ++t) {
        outer[t] = -1;
        if (t >= n) {
          L.c_gout[static_cast<size_t>(t) * NV + i] = L.c_gout[i];
          continue;
        }
        const int tr = m.v_tr[6 * static_cast<size_t>(c) + t] - 1;
        for (int q = 0; q < 3; ++q) {
          const int e = m.tr_ed[3 * static_cast<size_t>(tr) + q] - 1;
          if (m.ed_v[2 * static_cast<size_t>(e)] - 1 != c && m.ed_v[2 * static_cast<size_t>(e) + 1] - 1 != c)
            outer[t] = e;
        }
        if (outer[t] < 0) return off;
        L.c_gout[static_cast<size_t>(t) * NV + i] = L.edge_o2n[outer[t]];
      }
      if (n != 5 && n != 6) return off;
      for (int si = 0; si < n; ++si) {
        const int e = m.v_ed[6 * static_cast<size_t>(c) + si] - 1;
        for (int j = 0; j < n; ++j) {
          if (j == si) continue;
          const int k = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
          const int c3 = edge_connection(m, e, k);
          const int d = (j - si + n) % n;
          int want = -1;
          if (d == 1)
            want = outer[si];
          else if (d == n - 1)
            want = outer[j];
          else if (d == 2)
            want = m.v_ed[6 * static_cast<size_t>(c) + (si + 1) % n] - 1;
          else if (d == n - 2)
            want = m.v_ed[6 * static_cast<size_t>(c) + (si + n - 1) % n] - 1;
          if (c3 != want) return off;
        }
      }
      return std::string();
    });
    L.gass_cells = err.empty();
  }
  return "";
}

}  // namespace

std::string build_layout(const imodel_swm_mesh &m, const double *bt, Layout &L, int scheme,
                         int fsphere, double fcte) {
  const int nv = m.nv, ne = m.ne, nt = m.nt;
  std::string err;  // the first error of a parallel loop
  if (nv < 4 || ne < 6 || nt < 4) return "mesh sizes too small";
  if (!m.nnb || !m.v_ed || !m.v_tr || !m.hx_ttgout || !m.hx_tnrccw || !m.hx_areag ||
      !m.hx_trskw || !m.v_p || !m.ed_v || !m.ed_sh || !m.ed_leng || !m.edhx_leng ||
      !m.tr_v || !m.tr_ed || !m.tr_tg || !m.tr_areag || !m.tr_trhx_area || !m.tr_c_lat)
    return "mesh array pointer is NULL";
  if (!(m.erad > 0) || !(m.grav > 0)) return "erad and grav must be positive";
  err = par_for(nv, [&](int64_t i64) -> std::string {
    const int i = static_cast<int>(i64);
    int n = m.nnb[i];
    if (n < 3 || n > kMaxNb) return "nnb outside 3..6 at cell " + std::to_string(i + 1);
    for (int j = 0; j < n; ++j) {
      int e = m.v_ed[6 * static_cast<size_t>(i) + j];
      if (e < 1 || e > ne) return "v_ed index out of range at cell " + std::to_string(i + 1);
    }
    if (!(m.hx_areag[i] > 0)) return "non-positive hx_areag at cell " + std::to_string(i + 1);
    return std::string();
  });
  if (!err.empty()) return err;
  err = par_for(ne, [&](int64_t e64) -> std::string {
    const int e = static_cast<int>(e64);
    for (int s = 0; s < 2; ++s) {
      int c = m.ed_v[2 * static_cast<size_t>(e) + s], t = m.ed_sh[2 * static_cast<size_t>(e) + s];
      if (c < 1 || c > nv) return "ed_v index out of range at edge " + std::to_string(e + 1);
      if (t < 1 || t > nt) return "ed_sh index out of range at edge " + std::to_string(e + 1);
    }
    if (!(m.ed_leng[e] > 0)) return "non-positive ed_leng at edge " + std::to_string(e + 1);
    return std::string();
  });
  if (!err.empty()) return err;
  err = par_for(nt, [&](int64_t t64) -> std::string {
    const int t = static_cast<int>(t64);
    for (int s = 0; s < 3; ++s) {
      int c = m.tr_v[3 * static_cast<size_t>(t) + s], e = m.tr_ed[3 * static_cast<size_t>(t) + s];
      if (c < 1 || c > nv || e < 1 || e > ne)
        return "tr_v/tr_ed index out of range at triangle " + std::to_string(t + 1);
    }
    if (!(m.tr_areag[t] > 0)) return "non-positive tr_areag at triangle " + std::to_string(t + 1);
    return std::string();
  });
  if (!err.empty()) return err;

  L.nv = nv;
  L.ne = ne;
  L.nt = nt;
  L.erad = m.erad;
  L.grav = m.grav;
  L.omega = m.omega;

  // --- orderings ------------------------------------------------------
  {
    std::vector<uint64_t> key(nv);
    const int b = 20;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i) {
      const double *p = m.v_p + 3 * static_cast<size_t>(i);
      key[i] = hilbert3(quant(p[0], b), quant(p[1], b), quant(p[2], b), b);
    }
    sort_perm(L.cell_n2o, L.cell_o2n, key);
  }
  {
    std::vector<uint64_t> key(ne);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < ne; ++e) {
      uint64_t a = static_cast<uint64_t>(L.cell_o2n[m.ed_v[2 * static_cast<size_t>(e)] - 1]);
      uint64_t c = static_cast<uint64_t>(L.cell_o2n[m.ed_v[2 * static_cast<size_t>(e) + 1] - 1]);
      key[e] = (std::min(a, c) << 32) | std::max(a, c);
    }
    sort_perm(L.edge_n2o, L.edge_o2n, key);
  }
  {
    std::vector<uint64_t> key(nt);
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
      uint64_t v[3];
      for (int s = 0; s < 3; ++s)
        v[s] = static_cast<uint64_t>(L.cell_o2n[m.tr_v[3 * static_cast<size_t>(t) + s] - 1]);
      std::sort(v, v + 3);
      // (lowest, middle) vertex; the sort is stable, so the two triangles
      // of an edge keep the reference's order (no overflow below 2^32 cells)
      key[t] = (v[0] << 32) | v[1];
    }
    sort_perm(L.tri_n2o, L.tri_o2n, key);
  }

  // --- cells ----------------------------------------------------------
  const size_t NV = nv, NE = ne, NT = nt;
  fill(L.c_nnb, NV, 0);
  fill(L.c_ed, kMaxNb * NV, -1);
  fill(L.c_sd, kMaxNb * NV, 0.0);
  fill(L.c_div32, kMaxNb * NV, 0.0f);
  fill(L.c_kew32, kMaxNb * NV, 0.0f);
  L.c_areag.resize(NV);
  L.c_cellarea.resize(NV);
  fill(L.c_bt, NV, 0.0);
  fill(L.c_nb, kMaxNb * NV, 0);
  fill(L.c_tr, kMaxNb * NV, 0);
  fill(L.c_R32, kMaxNb * NV, 0.0f);
  fill(L.c_dg32, kMaxNb * NV, 0.0f);
  L.c_inva32.resize(NV);
  L.c_meta.resize(NV);
  if (nv >= (1 << 28)) return "more than 2^28 cells";
  err = par_for(nv, [&](int64_t i64) -> std::string {
    const int i = static_cast<int>(i64);
    const int c = L.cell_n2o[i];
    const int n = m.nnb[c];
    uint32_t tbits = 0;
    for (int j = 0; j < n; ++j) {
      const size_t q = 6 * static_cast<size_t>(c) + j;
      const int e = m.v_ed[q] - 1;
      // the neighbour across slot j is the other end of edge j
      const int a = m.ed_v[2 * static_cast<size_t>(e)] - 1, b = m.ed_v[2 * static_cast<size_t>(e) + 1] - 1;
      if (a != c && b != c) return "edge " + std::to_string(e + 1) + " does not touch cell " + std::to_string(c + 1);
      L.c_nb[j * NV + i] = L.cell_o2n[a == c ? b : a];
      const int t = m.v_tr[q] - 1;
      if (t < 0 || t >= nt) return "v_tr index out of range at cell " + std::to_string(c + 1);
      // edge j lies between triangles j-1 and j (smeshpack.f90:1071-1082)
      const int tp = m.v_tr[6 * static_cast<size_t>(c) + (j + n - 1) % n] - 1;
      const int s0 = m.ed_sh[2 * static_cast<size_t>(e)] - 1, s1 = m.ed_sh[2 * static_cast<size_t>(e) + 1] - 1;
      if (!((s0 == t && s1 == tp) || (s0 == tp && s1 == t)))
        return "v_tr order does not match v_ed at cell " + std::to_string(c + 1);
      L.c_tr[j * NV + i] = L.tri_o2n[t];
      L.c_R32[j * NV + i] = static_cast<float>(m.hx_hxtr_area[q]);
      L.c_dg32[j * NV + i] = static_cast<float>(m.hx_ttgout[q] * m.edhx_leng[e]);
      if (m.hx_tnrccw[q] < 0) tbits |= 1u << j;
    }
    L.c_meta[i] = static_cast<uint32_t>(n) | (tbits << 8);
    L.c_inva32[i] = static_cast<float>(1.0 / (m.hx_areag[c] * m.erad));
    return std::string();
  });
  if (!err.empty()) return err;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    const int c = L.cell_n2o[i];
    const int n = m.nnb[c];
    L.c_nnb[i] = static_cast<int8_t>(n);
    L.c_areag[i] = m.hx_areag[c];
    if (bt) L.c_bt[i] = bt[c];
    double cell_area = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
      cell_area = cell_area + 0.25 * m.ed_leng[e] * m.edhx_leng[e];
    }
    L.c_cellarea[i] = cell_area;
    for (int j = 0; j < n; ++j) {
      const int e = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
      const double s = static_cast<double>(m.hx_ttgout[6 * static_cast<size_t>(c) + j]);
      L.c_ed[j * NV + i] = L.edge_o2n[e];
      L.c_sd[j * NV + i] = s * m.edhx_leng[e];
      L.c_div32[j * NV + i] =
          static_cast<float>(s * m.edhx_leng[e] / (m.hx_areag[c] * m.erad));
      L.c_kew32[j * NV + i] =
          static_cast<float>(0.25 * m.ed_leng[e] * m.edhx_leng[e] / cell_area);
    }
  }

  // --- edges ----------------------------------------------------------
  L.e_v.resize(2 * NE);
  L.e_sh.resize(2 * NE);
  L.e_leng.resize(NE);
  L.e_dleng.resize(NE);
  L.e_kew.resize(NE);
  L.e_area.resize(NE);
  L.e_grad32.resize(NE);
  L.e_sgtg.resize(NE);
  L.e_gtg32.resize(NE);
  fill(L.e_nst, NE, 0);
  fill(L.e_stk, kMaxSt * NE, 0);
  fill(L.e_stw, kMaxSt * NE, 0.0);
  fill(L.e_stc32, kMaxSt * NE, 0.0f);
  if (scheme == IMODEL_SWM_GASS18) fill(L.e_stq, kMaxSt * NE, -1);
  fill(L.e_vs, 2 * NE, 0u);
  err = par_for(ne, [&](int64_t i64) -> std::string {
    const int i = static_cast<int>(i64);
    const int e = L.edge_n2o[i];
    for (int s = 0; s < 2; ++s) {
      L.e_v[s * NE + i] = L.cell_o2n[m.ed_v[2 * static_cast<size_t>(e) + s] - 1];
      L.e_sh[s * NE + i] = L.tri_o2n[m.ed_sh[2 * static_cast<size_t>(e) + s] - 1];
    }
    const double l = m.ed_leng[e], d = m.edhx_leng[e];
    L.e_leng[i] = l;
    L.e_dleng[i] = d;
    L.e_kew[i] = 0.25 * l * d;
    L.e_area[i] = l * d * 0.5;
    L.e_grad32[i] = static_cast<float>(1.0 / (l * m.erad));
    L.e_sgtg[i] = 0.0;  // 0 without ed%nr: the diffusion terms are then refused
    L.e_gtg32[i] = 0.0f;
    if (m.ed_nr) {
      // circumcentre directions of the edge's two triangles (only the sign
      // of nr . (c2 - c1) is used, and on a Delaunay mesh c2 - c1 runs
      // along the Voronoi edge, parallel to nr)
      double c[2][3];
      for (int s = 0; s < 2; ++s) circumcentre(m, m.ed_sh[2 * static_cast<size_t>(e) + s] - 1, c[s]);
      const double *nr = m.ed_nr + 3 * static_cast<size_t>(e);
      const double dot = nr[0] * (c[1][0] - c[0][0]) + nr[1] * (c[1][1] - c[0][1]) +
                         nr[2] * (c[1][2] - c[0][2]);
      const double sg = dot < 0 ? -1.0 : 1.0;  // dsign(1, x): +1 for x = +-0
      L.e_sgtg[i] = sg;
      L.e_gtg32[i] = static_cast<float>(sg / (d * m.erad));
    }
    // TRSK stencil, coriolis_ed order: cell ed%v(1) then ed%v(2), each in
    // its ccw edge order, the edge's own slot (zero weight) left out.
    int ns = 0;
    for (int s = 0; s < 2; ++s) {
      const int node = m.ed_v[2 * static_cast<size_t>(e) + s] - 1;
      const int n = m.nnb[node];
      int edcelli = -1;
      for (int j = 0; j < n; ++j)
        if (m.v_ed[6 * static_cast<size_t>(node) + j] - 1 == e) {
          edcelli = j;
          break;
        }
      if (edcelli < 0) return "edge " + std::to_string(e + 1) + " missing from its cell's edge list";
      L.e_vs[s * NE + i] = static_cast<uint32_t>(L.cell_o2n[node]) |
                           (static_cast<uint32_t>(edcelli) << 28);
      for (int j = 0; j < n; ++j) {
        if (j == edcelli) continue;
        if (ns >= kMaxSt) return "TRSK stencil longer than 10 at edge " + std::to_string(e + 1);
        const int k = m.v_ed[6 * static_cast<size_t>(node) + j] - 1;
        const double sc = std::copysign(
            1.0, 1.0 * m.hx_ttgout[6 * static_cast<size_t>(node) + j] *
                     m.hx_tnrccw[6 * static_cast<size_t>(node) + edcelli]);
        const double w = m.hx_trskw[36 * static_cast<size_t>(node) + 6 * static_cast<size_t>(j) + edcelli];
        L.e_stk[ns * NE + i] = L.edge_o2n[k];
        if (scheme == IMODEL_SWM_GASS18) {
          const int c3 = edge_connection(m, e, k);
          L.e_stq[ns * NE + i] = c3 < 0 ? -1 : L.edge_o2n[c3];
        }
        L.e_stw[ns * NE + i] = w * sc;
        L.e_stc32[ns * NE + i] = static_cast<float>(0.5 * w * sc * m.edhx_leng[k] / l);
        ++ns;
      }
    }
    L.e_nst[i] = static_cast<int8_t>(ns);
    return std::string();
  });
  if (!err.empty()) return err;

  // packed cell slots and edge cell words for vector loads
  fill(L.c_pk, kMaxNb * NV * 4, 0);
  fill(L.c_kd, kMaxNb * NV * 2, 0.0f);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    const int n = L.c_nnb[i];
    for (int j = 0; j < kMaxNb; ++j) {
      const int src = j < n ? j : 0;  // padding repeats slot 0 ...
      const size_t q = (static_cast<size_t>(j) * NV + i);
      L.c_pk[4 * q + 0] = L.c_ed[src * NV + i];
      L.c_pk[4 * q + 1] = L.c_nb[src * NV + i];
      L.c_pk[4 * q + 2] = L.c_tr[src * NV + i];
      float r = j < n ? L.c_R32[src * NV + i] : 0.0f;  // ... with zero weights
      int32_t rb;
      std::memcpy(&rb, &r, sizeof(rb));
      L.c_pk[4 * q + 3] = rb;
      L.c_kd[2 * q + 0] = j < n ? L.c_kew32[src * NV + i] : 0.0f;
      L.c_kd[2 * q + 1] = j < n ? L.c_dg32[src * NV + i] : 0.0f;
    }
  }
  L.e_vs2.resize(2 * NE);
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < NE; ++e) {
    L.e_vs2[2 * e] = L.e_vs[e];
    L.e_vs2[2 * e + 1] = L.e_vs[NE + e];
  }

  // --- triangles ------------------------------------------------------
  L.t_ed.resize(3 * NT);
  L.t_v.resize(3 * NT);
  L.t_lt.resize(3 * NT);
  L.t_kite.resize(3 * NT);
  L.t_circ32.resize(3 * NT);
  L.t_kite32.resize(3 * NT);
  L.t_areag.resize(NT);
  L.t_f.resize(NT);
  L.t_f32.resize(NT);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nt; ++i) {
    const int t = L.tri_n2o[i];
    const double A = m.tr_areag[t];
    L.t_areag[i] = A;
    // vort_tr's Coriolis parameter (swm_operators.f90:592-601): 2.*Omega*
    // dsin(lat) (fsphere 0) or the constant fcte (fsphere 2)
    L.t_f[i] = fsphere == 2 ? fcte : 2.0 * m.omega * std::sin(m.tr_c_lat[t]);
    L.t_f32[i] = static_cast<float>(L.t_f[i]);
    for (int s = 0; s < 3; ++s) {
      const int e = m.tr_ed[3 * static_cast<size_t>(t) + s] - 1;
      const int v = m.tr_v[3 * static_cast<size_t>(t) + s] - 1;
      const double tg = static_cast<double>(m.tr_tg[3 * static_cast<size_t>(t) + s]);
      L.t_ed[s * NT + i] = L.edge_o2n[e];
      L.t_v[s * NT + i] = L.cell_o2n[v];
      L.t_lt[s * NT + i] = m.ed_leng[e] * tg;
      L.t_kite[s * NT + i] = m.tr_trhx_area[3 * static_cast<size_t>(t) + s];
      L.t_circ32[s * NT + i] = static_cast<float>(m.ed_leng[e] * tg / (A * m.erad));
      L.t_kite32[s * NT + i] = static_cast<float>(m.tr_trhx_area[3 * static_cast<size_t>(t) + s] / A);
    }
  }

  // --- APVM points (need ed%nr for grad_tr2ed's sign) --------------------
  if (m.ed_nr && m.ed_c) {
    L.t_c.resize(3 * NT);
    L.e_c.resize(3 * NE);
    L.c_p.resize(3 * NV);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nt; ++i) {
      double c[3];
      circumcentre(m, L.tri_n2o[i], c);
      for (int k = 0; k < 3; ++k) L.t_c[k * NT + i] = c[k];
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i)
      for (int k = 0; k < 3; ++k) L.e_c[k * NE + i] = m.ed_c[3 * static_cast<size_t>(L.edge_n2o[i]) + k];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i)
      for (int k = 0; k < 3; ++k) L.c_p[k * NV + i] = m.v_p[3 * static_cast<size_t>(L.cell_n2o[i]) + k];
    fill(L.t_apw32, 9 * NT, 0.0f);
    fill(L.t_cc32, 3 * NT, 0.0f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nt; ++i) {
      const int t = L.tri_n2o[i];
      for (int s = 0; s < 3; ++s) {
        const int e = m.tr_ed[3 * static_cast<size_t>(t) + s] - 1;
        const double sg = -static_cast<double>(m.tr_tg[3 * static_cast<size_t>(t) + s]);
        for (int k = 0; k < 3; ++k) {
          const double d = m.ed_c[3 * static_cast<size_t>(e) + k] - L.t_c[k * NT + i];
          L.t_apw32[(3 * s + k) * NT + i] = static_cast<float>(sg * d * m.ed_leng[e] / m.tr_areag[t]);
        }
      }
      for (int k = 0; k < 3; ++k) L.t_cc32[k * NT + i] = static_cast<float>(L.t_c[k * NT + i]);
    }
    fill(L.c_apw32, 18 * NV, 0.0f);
    fill(L.c_p32, 3 * NV, 0.0f);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i) {
      const int c = L.cell_n2o[i];
      for (int j = 0; j < m.nnb[c]; ++j) {
        const int e = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
        const double sg = static_cast<double>(m.hx_ttgout[6 * static_cast<size_t>(c) + j]);
        for (int k = 0; k < 3; ++k) {
          const double d = m.ed_c[3 * static_cast<size_t>(e) + k] - L.c_p[k * NV + i];
          L.c_apw32[(3 * j + k) * NV + i] = static_cast<float>(sg * d * m.edhx_leng[e] / m.hx_areag[c]);
        }
      }
      for (int k = 0; k < 3; ++k) L.c_p32[k * NV + i] = static_cast<float>(L.c_p[k * NV + i]);
    }
  }
  // --- geometry of the pxt16, gass18 and dtred branches -------------------
  if (scheme != IMODEL_SWM_TRSK10) {
    if (scheme < IMODEL_SWM_TRSK10 || scheme > IMODEL_SWM_DTRED) return "unknown scheme";
    if (!m.ed_nr || !m.ed_c) return "the pxt16, gass18 and dtred schemes need ed_nr and ed_c";
    if (scheme == IMODEL_SWM_PXT16) {
      L.t_bary.resize(3 * NT);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < nt; ++i) {
        const int t = L.tri_n2o[i];
        const double pc[3] = {L.t_c[i], L.t_c[NT + i], L.t_c[2 * NT + i]};
        const double *p[3];
        for (int k = 0; k < 3; ++k)
          p[k] = m.v_p + 3 * static_cast<size_t>(m.tr_v[3 * static_cast<size_t>(t) + k] - 1);
        const double b[3] = {std::fabs(det3(pc, p[1], p[2])), std::fabs(det3(pc, p[2], p[0])),
                             std::fabs(det3(pc, p[0], p[1]))};
        double area = b[0];
        area = area + b[1];
        area = area + b[2];
        for (int k = 0; k < 3; ++k) L.t_bary[k * NT + i] = b[k] / area;
      }
    }
    if (scheme == IMODEL_SWM_PXT16 || scheme == IMODEL_SWM_DTRED) {
      L.e_dist.resize(2 * NE);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < ne; ++i) {
        const int e = L.edge_n2o[i];
        for (int s = 0; s < 2; ++s) {
          const int ti = L.e_sh[s * NE + i];
          const double c[3] = {L.t_c[ti], L.t_c[NT + ti], L.t_c[2 * NT + ti]};
          L.e_dist[s * NE + i] = arclen(m.ed_c + 3 * static_cast<size_t>(e), c);
        }
      }
    }
    if (scheme == IMODEL_SWM_GASS18) {
      L.t_edarea.resize(3 * NT);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < nt; ++i) {
        const int t = L.tri_n2o[i];
        const double pc[3] = {L.t_c[i], L.t_c[NT + i], L.t_c[2 * NT + i]};
        for (int s = 0; s < 3; ++s) {
          const int e = m.tr_ed[3 * static_cast<size_t>(t) + s] - 1;
          L.t_edarea[s * NT + i] =
              sphtriarea(pc, m.v_p + 3 * static_cast<size_t>(m.ed_v[2 * static_cast<size_t>(e)] - 1),
                         m.v_p + 3 * static_cast<size_t>(m.ed_v[2 * static_cast<size_t>(e) + 1] - 1));
        }
      }
    }
    L.e_nr.resize(3 * NE);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ne; ++i)
      for (int k = 0; k < 3; ++k) L.e_nr[k * NE + i] = m.ed_nr[3 * static_cast<size_t>(L.edge_n2o[i]) + k];
    const std::string msg = scheme_fp32(m, L, scheme);
    if (!msg.empty()) return msg;
  }
  L.t_recA.resize(4 * NT);
  L.t_recB.resize(4 * NT);
  L.t_recC.resize(4 * NT);
  auto bits = [](float f) {
    int32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return b;
  };
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < NT; ++i) {
    int32_t *a = &L.t_recA[4 * i], *b = &L.t_recB[4 * i], *c = &L.t_recC[4 * i];
    a[0] = L.t_ed[i];
    a[1] = L.t_ed[NT + i];
    a[2] = L.t_ed[2 * NT + i];
    a[3] = L.t_v[i];
    b[0] = L.t_v[NT + i];
    b[1] = L.t_v[2 * NT + i];
    b[2] = bits(L.t_circ32[i]);
    b[3] = bits(L.t_circ32[NT + i]);
    c[0] = bits(L.t_circ32[2 * NT + i]);
    c[1] = bits(L.t_kite32[i]);
    c[2] = bits(L.t_kite32[NT + i]);
    c[3] = bits(L.t_kite32[2 * NT + i]);
  }
  {
    // 16-bit triangle records: bases per warp of 32 triangles
    const size_t nw = (NT + 31) / 32;
    fill(L.t_c16A, 4 * NT, 0u);
    fill(L.t_c16B, 4 * NT, 0.0f);
    fill(L.t_c16C, 2 * NT, 0.0f);
    fill(L.t_wb, 2 * nw, 0);
#pragma omp parallel for schedule(static)
    for (size_t w = 0; w < nw; ++w) {
      const size_t t0 = 32 * w, t1 = std::min(NT, t0 + 32);
      int32_t lo[2] = {INT32_MAX, INT32_MAX}, hi[2] = {INT32_MIN, INT32_MIN};
      for (size_t t = t0; t < t1; ++t)
        for (int s = 0; s < 3; ++s) {
          lo[0] = std::min(lo[0], L.t_ed[s * NT + t]);
          hi[0] = std::max(hi[0], L.t_ed[s * NT + t]);
          lo[1] = std::min(lo[1], L.t_v[s * NT + t]);
          hi[1] = std::max(hi[1], L.t_v[s * NT + t]);
        }
      const bool ok = static_cast<int64_t>(hi[0]) - lo[0] <= 0xFFFF &&
                      static_cast<int64_t>(hi[1]) - lo[1] <= 0xFFFF;
      L.t_wb[2 * w] = ok ? lo[0] : 0;
      L.t_wb[2 * w + 1] = ok ? lo[1] : -1;
      for (size_t t = t0; t < t1; ++t) {
        uint32_t oe[3] = {0u, 0u, 0u}, ov[3] = {0u, 0u, 0u};
        if (ok)
          for (int s = 0; s < 3; ++s) {
            oe[s] = static_cast<uint32_t>(L.t_ed[s * NT + t] - lo[0]);
            ov[s] = static_cast<uint32_t>(L.t_v[s * NT + t] - lo[1]);
          }
        uint32_t *a = &L.t_c16A[4 * t];
        a[0] = oe[0] | (oe[1] << 16);
        a[1] = oe[2] | (ov[0] << 16);
        a[2] = ov[1] | (ov[2] << 16);
        a[3] = static_cast<uint32_t>(bits(L.t_circ32[t]));
        float *b = &L.t_c16B[4 * t];
        b[0] = L.t_circ32[NT + t];
        b[1] = L.t_circ32[2 * NT + t];
        b[2] = L.t_kite32[t];
        b[3] = L.t_kite32[NT + t];
        L.t_c16C[2 * t] = L.t_kite32[2 * NT + t];
        L.t_c16C[2 * t + 1] = L.t_f32[t];
      }
    }
  }
  return "";
}

}  // namespace imodel

namespace imodel {

uint16_t bf16_bits(float v) {
  uint32_t b;
  std::memcpy(&b, &v, sizeof(b));
  if ((b & 0x7F800000u) == 0x7F800000u && (b & 0x007FFFFFu)) return static_cast<uint16_t>(b >> 16);
  const uint64_t r = (static_cast<uint64_t>(b) + 0x7FFFu + ((b >> 16) & 1u)) >> 16;
  return static_cast<uint16_t>(r & 0xFFFFu);
}

// Same inputs as imodel_gb300/learned.py (stencil, geometry_features): for
// each edge and each of its two cells ed%v(1), ed%v(2), the cell's other
// edges counter-clockwise from the edge (5 slots per cell, the sixth slot of
// a pentagon empty), with sign ttgout_c(j) * tnrccw_c(i_e) and TRSK weight
// trskw_c(i_e, j); geometry centred on a regular hexagonal grid and scaled:
// 10 (l_e / mean l - 1), 10 (d_e / l_e - 1/sqrt 3), 10 (A_c / (l_e d_e) - 3/2)
// for both cells and 20 (w - (r/n - 1/2)) for the 10 weights.
std::string build_learned_layout(const imodel_swm_mesh &m, const Layout &L, LearnedLayout &LL) {
  const int ne = m.ne;
  constexpr int T = LearnedLayout::kTile;
  LL.ntiles = (static_cast<int64_t>(ne) + T - 1) / T;
  fill(LL.blocks, static_cast<size_t>(LL.ntiles) * LearnedLayout::kBlockBytes, 0);
  // entry k of array `off` (element size `sz`) in the block of device edge i
  auto at = [&](int64_t i, int off, int k, int sz) -> uint8_t * {
    return LL.blocks.data() + (i / T) * LearnedLayout::kBlockBytes + off +
           static_cast<size_t>(k) * sz;
  };
  auto put_i32 = [&](int64_t i, int off, int k, int32_t v) {
    std::memcpy(at(i, off, k, 4), &v, 4);
  };
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < ne; ++i) {
    const int64_t r = i % T;
    put_i32(i, LearnedLayout::kEsh, static_cast<int>(r), L.e_sh[i]);
    put_i32(i, LearnedLayout::kEsh, static_cast<int>(T + r), L.e_sh[static_cast<size_t>(ne) + i]);
    const uint32_t w[2] = {L.e_vs2[2 * i], L.e_vs2[2 * i + 1]};
    std::memcpy(at(i, LearnedLayout::kEvs, static_cast<int>(r), 8), w, 8);
  }
  double lmean = 0.0;
  for (int e = 0; e < ne; ++e) lmean += m.ed_leng[e];
  lmean /= ne;
  return par_for(ne, [&](int64_t e64) -> std::string {
    const int e = static_cast<int>(e64);
    const int i = L.edge_o2n[e];
    const int r = i % T;
    const double l = m.ed_leng[e], d = m.edhx_leng[e];
    float g[14];
    g[0] = static_cast<float>(10.0 * (l / lmean - 1.0));
    g[1] = static_cast<float>(10.0 * (d / l - 1.0 / std::sqrt(3.0)));
    for (int side = 0; side < 2; ++side) {
      const int c = m.ed_v[2 * static_cast<size_t>(e) + side] - 1;
      const int n = m.nnb[c];
      g[2 + side] = static_cast<float>(10.0 * (m.hx_areag[c] / (l * d) - 1.5));
      int slot = -1;
      for (int j = 0; j < n; ++j)
        if (m.v_ed[6 * static_cast<size_t>(c) + j] - 1 == e) slot = j;
      if (slot < 0) return "edge missing from its cell's edge list";
      for (int q = 1; q < 6; ++q) {
        const int col = side * 5 + (q - 1);
        float w = 0.0f;
        if (q < n) {
          const int j = (slot + q) % n;
          const int k = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
          const int s = m.hx_ttgout[6 * static_cast<size_t>(c) + j] *
                        m.hx_tnrccw[6 * static_cast<size_t>(c) + slot];
          put_i32(i, LearnedLayout::kLst, col * T + r, (s < 0 ? -1 : 1) * (L.edge_o2n[k] + 1));
          const double wreg = static_cast<double>(q) / n - 0.5;
          w = static_cast<float>(
              20.0 * (m.hx_trskw[36 * static_cast<size_t>(c) + 6 * static_cast<size_t>(j) + slot] -
                      wreg));
        }
        g[4 + col] = w;
      }
    }
    for (int q = 0; q < 14; ++q) {
      const uint16_t b16 = bf16_bits(g[q]);
      std::memcpy(at(i, LearnedLayout::kGeo, 16 * r + q, 2), &b16, 2);
    }
    return std::string();
  });
}

std::string build_weight_arrays(const imodel_swm_mesh &m, const Layout &L, WeightArrays &W) {
  const int nv = L.nv, ne = L.ne;
  const size_t NV = nv, NE = ne;
  if (m.nv != nv || m.ne != ne) return "mesh sizes differ from the layout's";
  fill(W.e_stw, kMaxSt * NE, 0.0);
  fill(W.e_stc32, kMaxSt * NE, 0.0f);
  // the TRSK stencil slots in build_layout's order (cells ed%v(1), ed%v(2),
  // each ccw, the edge's own slot left out)
  std::string err = par_for(ne, [&](int64_t i64) -> std::string {
    const int i = static_cast<int>(i64);
    const int e = L.edge_n2o[i];
    const double l = m.ed_leng[e];
    int ns = 0;
    for (int s = 0; s < 2; ++s) {
      const int node = m.ed_v[2 * static_cast<size_t>(e) + s] - 1;
      const int n = m.nnb[node];
      int edcelli = -1;
      for (int j = 0; j < n; ++j)
        if (m.v_ed[6 * static_cast<size_t>(node) + j] - 1 == e) {
          edcelli = j;
          break;
        }
      if (edcelli < 0) return "edge " + std::to_string(e + 1) + " missing from its cell's edge list";
      for (int j = 0; j < n; ++j) {
        if (j == edcelli) continue;
        const int k = m.v_ed[6 * static_cast<size_t>(node) + j] - 1;
        if (ns >= kMaxSt || L.e_stk[ns * NE + i] != L.edge_o2n[k])
          return "the mesh's stencil differs from the layout's at edge " + std::to_string(e + 1);
        const double sc = std::copysign(
            1.0, 1.0 * m.hx_ttgout[6 * static_cast<size_t>(node) + j] *
                     m.hx_tnrccw[6 * static_cast<size_t>(node) + edcelli]);
        const double w = m.hx_trskw[36 * static_cast<size_t>(node) + 6 * static_cast<size_t>(j) + edcelli];
        W.e_stw[ns * NE + i] = w * sc;
        W.e_stc32[ns * NE + i] = static_cast<float>(0.5 * w * sc * m.edhx_leng[k] / l);
        ++ns;
      }
    }
    return std::string();
  });
  if (!err.empty()) return err;
  fill(W.c_R32, kMaxNb * NV, 0.0f);
  W.c_pk = L.c_pk;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    const int c = L.cell_n2o[i];
    const int n = m.nnb[c];
    for (int j = 0; j < n; ++j)
      W.c_R32[j * NV + i] = static_cast<float>(m.hx_hxtr_area[6 * static_cast<size_t>(c) + j]);
    for (int j = 0; j < kMaxNb; ++j) {
      const int src = j < n ? j : 0;
      const float r = j < n ? W.c_R32[src * NV + i] : 0.0f;
      int32_t rb;
      std::memcpy(&rb, &r, sizeof(rb));
      W.c_pk[4 * (static_cast<size_t>(j) * NV + i) + 3] = rb;
    }
  }
  return "";
}

// ---- learned TRSK weights ----------------------------------------------------
std::string build_kite_inputs(const imodel_swm_mesh &m, KiteInputs &K) {
  const int nv = m.nv;
  if (!m.v_p || !m.v_tr || !m.tr_v || !m.hx_hxtr_area)
    return "the learned weights need v_p, v_tr and tr_v";
  size_t nrow = 0;
  for (int c = 0; c < nv; ++c) nrow += static_cast<size_t>(m.nnb[c]);
  // every row is written in full by the loop below
  K.x.resize(nrow * 24);
  K.cell.resize(nrow);
  K.slot.resize(nrow);
  // row of (c, j): slot-major, the cells with nnb > j in order
  std::vector<size_t> row_of(6 * static_cast<size_t>(nv), 0);
  {
    size_t acc = 0;
    for (int j = 0; j < 6; ++j)
      for (int c = 0; c < nv; ++c)
        if (m.nnb[c] > j) row_of[6 * static_cast<size_t>(c) + j] = acc++;
  }
  auto tangent = [](const double *v, const double *p, double *t) {
    const double vp = dot3(v, p);
    for (int k = 0; k < 3; ++k) t[k] = v[k] - vp * p[k];
  };
  static const int kDj[6] = {0, -1, 1, -2, 2, 3};
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nv; ++c) {
    const int n = m.nnb[c];
    const double *P = m.v_p + 3 * static_cast<size_t>(c);
    const double sA = std::sqrt(m.hx_areag[c]);
    const double *R = m.hx_hxtr_area + 6 * static_cast<size_t>(c);
    double T[6][3], Tt[6][3], r[6], V[3] = {0.0, 0.0, 0.0};
    double sum_d = 0.0, sum_l = 0.0, sum_r = 0.0;
    int ed[6];
    for (int j = 0; j < n; ++j) {
      circumcentre(m, m.v_tr[6 * static_cast<size_t>(c) + j] - 1, T[j]);
      for (int k = 0; k < 3; ++k) V[k] += T[j][k];
      tangent(T[j], P, Tt[j]);
      r[j] = std::sqrt(dot3(Tt[j], Tt[j]));
      ed[j] = m.v_ed[6 * static_cast<size_t>(c) + j] - 1;
      sum_d += m.edhx_leng[ed[j]];
      sum_l += m.ed_leng[ed[j]];
      sum_r += r[j];
    }
    for (int k = 0; k < 3; ++k) V[k] /= n;
    double O[3];
    tangent(V, P, O);
    const double mean_d = sum_d / n, mean_l = sum_l / n, mean_r = sum_r / n;
    for (int j = 0; j < n; ++j) {
      double f[24] = {};
      for (int q = 0; q < 6; ++q) f[q] = 10.0 * (R[((j + kDj[q]) % n + n) % n] - 1.0 / n);
      f[6] = n == 5 ? 1.0 : 0.0;
      const double dn = std::sqrt(dot3(Tt[j], Tt[j]));
      const double D[3] = {Tt[j][0] / dn, Tt[j][1] / dn, Tt[j][2] / dn};
      const double Q[3] = {P[1] * D[2] - P[2] * D[1], P[2] * D[0] - P[0] * D[2],
                           P[0] * D[1] - P[1] * D[0]};
      f[7] = 10.0 * dot3(O, D) / sA;
      f[8] = 10.0 * dot3(O, Q) / sA;
      const int e0 = ed[j], e1 = ed[(j + 1) % n];
      f[9] = 10.0 * (m.edhx_leng[e0] / mean_d - 1.0);
      f[10] = 10.0 * (m.edhx_leng[e1] / mean_d - 1.0);
      f[11] = 10.0 * (m.ed_leng[e0] / mean_l - 1.0);
      f[12] = 10.0 * (m.ed_leng[e1] / mean_l - 1.0);
      f[13] = 10.0 * (r[j] / mean_r - 1.0);
      const size_t row = row_of[6 * static_cast<size_t>(c) + j];
      for (int q = 0; q < 24; ++q) K.x[24 * row + q] = bf16_bits(static_cast<float>(f[q]));
      K.cell[row] = c;
      K.slot[row] = static_cast<int8_t>(j);
    }
  }
  return "";
}

void apply_kite_outputs(const imodel_swm_mesh &m, const KiteInputs &K, const float *y,
                        HVec<double> &hxtr, HVec<double> &trskw) {
  const int nv = m.nv;
  HVec<double> dR;
  fill(dR, 6 * static_cast<size_t>(nv), 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < static_cast<int64_t>(K.cell.size()); ++r)
    dR[6 * static_cast<size_t>(K.cell[r]) + K.slot[r]] = 0.1 * static_cast<double>(y[r]);
  hxtr.resize(6 * static_cast<size_t>(nv));
  {
    const int64_t n6 = 6 * static_cast<int64_t>(nv);
    double *d = hxtr.data();
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n6; ++q) d[q] = m.hx_hxtr_area[q];
  }
  fill(trskw, 36 * static_cast<size_t>(nv), 0.0);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nv; ++c) {
    const int n = m.nnb[c];
    double *R = hxtr.data() + 6 * static_cast<size_t>(c);
    const double *d = dR.data() + 6 * static_cast<size_t>(c);
    double mean = 0.0;
    for (int j = 0; j < n; ++j) mean += d[j];
    mean /= n;
    for (int j = 0; j < n; ++j) R[j] += d[j] - mean;
    // calc_trisk_weights: w(i, j) = sum_{k=i}^{j-1} R(k) - 1/2, cyclic
    double *w = trskw.data() + 36 * static_cast<size_t>(c);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        if (i == j) continue;
        double s = 0.0;
        if (j < i) {
          for (int k = i; k < n; ++k) s = s + R[k];
          for (int k = 0; k < j; ++k) s = s + R[k];
        } else {
          for (int k = i; k < j; ++k) s = s + R[k];
        }
        w[6 * j + i] = s - 0.5;
      }
  }
}

}  // namespace imodel

// ---- test hook: a digest of the whole layout ---------------------------------

namespace {

uint64_t fnv1a(const void *p, size_t n, uint64_t h) {
  const unsigned char *c = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
  return h;
}
template <class V>
uint64_t digest_of(const V &v, uint64_t h) {
  h = fnv1a(v.data(), v.size() * sizeof(typename V::value_type), h);
  const uint64_t n = v.size();
  return fnv1a(&n, sizeof(n), h);
}

}  // namespace

extern "C" int imodel_swm_test_layout_digest(const imodel_swm_mesh *m, int32_t scheme,
                                             int32_t nthreads, uint64_t *digest) {
  if (!m || !digest || nthreads < 0) return IMODEL_SWM_EINVAL;
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  imodel::Layout L;
  std::string msg;
  try {
    msg = imodel::build_layout(*m, nullptr, L, scheme, 0, 0.0);
  } catch (const std::bad_alloc &) {
    msg = "host allocation failed";
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  if (!msg.empty()) return IMODEL_SWM_EINVAL;
  uint64_t h = 1469598103934665603ull;
#define IMODEL_DIGEST(f) h = digest_of(L.f, h);
  IMODEL_DIGEST(cell_n2o) IMODEL_DIGEST(cell_o2n) IMODEL_DIGEST(edge_n2o) IMODEL_DIGEST(edge_o2n)
  IMODEL_DIGEST(tri_n2o) IMODEL_DIGEST(tri_o2n) IMODEL_DIGEST(c_nnb) IMODEL_DIGEST(c_ed)
  IMODEL_DIGEST(c_sd) IMODEL_DIGEST(c_areag) IMODEL_DIGEST(c_cellarea) IMODEL_DIGEST(c_bt)
  IMODEL_DIGEST(c_div32) IMODEL_DIGEST(c_kew32) IMODEL_DIGEST(c_nb) IMODEL_DIGEST(c_tr)
  IMODEL_DIGEST(c_R32) IMODEL_DIGEST(c_dg32) IMODEL_DIGEST(c_inva32) IMODEL_DIGEST(c_meta)
  IMODEL_DIGEST(e_vs) IMODEL_DIGEST(c_pk) IMODEL_DIGEST(c_kd) IMODEL_DIGEST(e_vs2)
  IMODEL_DIGEST(e_v) IMODEL_DIGEST(e_sh) IMODEL_DIGEST(e_leng) IMODEL_DIGEST(e_dleng)
  IMODEL_DIGEST(e_kew) IMODEL_DIGEST(e_grad32) IMODEL_DIGEST(e_sgtg) IMODEL_DIGEST(e_gtg32)
  IMODEL_DIGEST(e_nst) IMODEL_DIGEST(e_stk) IMODEL_DIGEST(e_stw) IMODEL_DIGEST(e_stc32)
  IMODEL_DIGEST(t_ed) IMODEL_DIGEST(t_v) IMODEL_DIGEST(t_lt) IMODEL_DIGEST(t_kite)
  IMODEL_DIGEST(t_areag) IMODEL_DIGEST(t_f) IMODEL_DIGEST(e_c) IMODEL_DIGEST(t_c)
  IMODEL_DIGEST(c_p) IMODEL_DIGEST(t_apw32) IMODEL_DIGEST(t_cc32) IMODEL_DIGEST(c_apw32)
  IMODEL_DIGEST(c_p32) IMODEL_DIGEST(t_recA) IMODEL_DIGEST(t_recB) IMODEL_DIGEST(t_recC)
  IMODEL_DIGEST(t_c16A) IMODEL_DIGEST(t_c16B) IMODEL_DIGEST(t_c16C) IMODEL_DIGEST(t_wb)
  IMODEL_DIGEST(t_circ32) IMODEL_DIGEST(t_kite32) IMODEL_DIGEST(t_f32) IMODEL_DIGEST(e_area)
  IMODEL_DIGEST(t_bary) IMODEL_DIGEST(e_dist) IMODEL_DIGEST(t_edarea) IMODEL_DIGEST(e_nr)
  IMODEL_DIGEST(e_stq) IMODEL_DIGEST(e_qw32) IMODEL_DIGEST(e_dtc32) IMODEL_DIGEST(c_C32) IMODEL_DIGEST(c_gout) IMODEL_DIGEST(c_qw32)
  IMODEL_DIGEST(t_dpa32) IMODEL_DIGEST(t_dopp) IMODEL_DIGEST(e_nr32) IMODEL_DIGEST(e_dw32)
#undef IMODEL_DIGEST
  *digest = h;
  return IMODEL_SWM_OK;
}
