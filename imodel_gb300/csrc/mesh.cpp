// Icosahedral Voronoi/Delaunay grid builder (host C++).
//
// Restates the geometry of iModel's smeshpack for non-optimised hierarchical
// icosahedral grids (meshbuild with kind=icos, hrchy>0, optm=nopt;
// src/smeshpack.f90:77-368) and the TRSK precomputation of
// initialize_gridprop (src/swm.f90:979-992).  Every per-entity value follows
// the reference's arithmetic step by step (same operand order, no FMA
// contraction: build with -ffp-contract=off) so that the fields handed to the
// time step are the reference's fields.
//
// Topology: the reference triangulates each level with STRIPACK; for nodes
// appended at edge midpoints that Delaunay triangulation is the 4-way
// subdivision of the previous level, which is what this builder constructs.
// delaunay_check() verifies the empty-circumcircle property on every edge.

#include "imodel_mesh.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// constants.f90:31 -- pi is built from a default-real (float) literal.
const double kPi = 4.0 * static_cast<double>(0.78539816339744830961566f);
// constants.f90:45 -- eps = epsilon(1.) (single precision epsilon).
const double kEps = static_cast<double>(1.1920928955078125e-07f);

struct V3 {
  double x, y, z;
};
inline V3 sub(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(const V3 &a, const V3 &b) {
  double s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
// smeshpack.f90:6560-6578
inline V3 cross(const V3 &a, const V3 &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// smeshpack.f90:7061-7073
inline double norm(const V3 &p) { return std::sqrt(dot(p, p)); }
inline V3 divs(const V3 &p, double s) { return {p.x / s, p.y / s, p.z / s}; }
inline V3 muls(const V3 &p, double s) { return {p.x * s, p.y * s, p.z * s}; }
// smeshpack.f90:6580-6596
inline double det3(const V3 &a, const V3 &b, const V3 &c) { return dot(cross(a, b), c); }

// arclen, smeshpack.f90:4624-4657
double arclen(const V3 &p, const V3 &q) {
  V3 s = {p.x + q.x, p.y + q.y, p.z + q.z};
  double d = dot(s, s);
  if (d == 0.0) return kPi;
  if (d >= 4.0) return 0.0;
  return 2.0 * std::atan(std::sqrt((4.0 - d) / d));
}

// trcircumc, smeshpack.f90:4659-4687
V3 trcircumc(const V3 &p1, const V3 &p2, const V3 &p3) {
  const double tol = kEps / 100.0;
  if (norm(sub(p1, p2)) < tol || norm(sub(p2, p3)) < tol || norm(sub(p1, p3)) < tol)
    return {0.0, 0.0, 0.0};
  V3 cp = cross(sub(p2, p1), sub(p3, p1));
  return divs(cp, norm(cp));
}

// sphtriarea (L'Huilier), smeshpack.f90:4710-4762
double sphtriarea(const V3 &p1, const V3 &p2, const V3 &p3) {
  const double tol = kEps / 100.0;
  if (norm(sub(p1, p2)) < tol || norm(sub(p2, p3)) < tol || norm(sub(p1, p3)) < tol)
    return 0.0;
  double a = arclen(p1, p2);
  double b = arclen(p2, p3);
  double c = arclen(p3, p1);
  double s = (a + b + c) / 2.0;
  double tmp = std::tan(s / 2.0) * std::tan((s - a) / 2.0);
  tmp = tmp * std::tan((s - b) / 2.0);
  tmp = tmp * std::tan((s - c) / 2.0);
  if (tmp < 0.0) return 0.0;
  return 4.0 * std::atan(std::sqrt(tmp));
}

// cart2sph, smeshpack.f90:4279-4313
void cart2sph(double x, double y, double z, double &lon, double &lat) {
  double pnrm = std::sqrt(x * x + y * y + z * z);
  lon = (x != 0.0 || y != 0.0) ? std::atan2(y, x) : 0.0;
  lat = (pnrm != 0.0) ? std::asin(z / pnrm) : 0.0;
}

// sph2cart, smeshpack.f90:4251-4277
V3 sph2cart(double lon, double lat) {
  double coslat = std::cos(lat);
  return {coslat * std::cos(lon), coslat * std::sin(lon), std::sin(lat)};
}

// midpoint_ed / midpoint_edhx, smeshpack.f90:6286-6334
V3 midpoint(const V3 &a, const V3 &b) {
  V3 p = {(a.x + b.x) / 2.0, (a.y + b.y) / 2.0, (a.z + b.z) / 2.0};
  return divs(p, norm(p));
}

// icosanodes0, smeshpack.f90:1197-1280
std::vector<V3> icosanodes0(int pos) {
  std::vector<V3> p(12);
  if (pos == 0) {  // eqs
    const double radius = 1.0;
    const double sqrt5 = std::sqrt(5.0);
    const double phi = (1.0 + sqrt5) * 0.5;
    const double ratio = std::sqrt(10.0 + (2.0 * sqrt5)) / (4.0 * phi);
    const double a = (radius / ratio) * 0.5;
    const double b = (radius / ratio) / (2.0 * phi);
    p[0] = {0, b, -a};
    p[1] = {0, -b, -a};
    p[2] = {a, 0, -b};
    p[3] = {-a, 0, -b};
    p[4] = {b, a, 0};
    p[5] = {-b, a, 0};
    p[6] = {-a, 0, b};
    p[7] = {a, 0, b};
    p[8] = {b, -a, 0};
    p[9] = {-b, -a, 0};
    p[10] = {0, b, a};
    p[11] = {0, -b, a};
  } else {  // pol
    p[0] = {0, 0, 1};
    double lat = std::atan(0.5);
    // dlon = 2/5.*pi : the quotient is a default-real (float) 0.4
    const double dlon = static_cast<double>(2.0f / 5.0f) * kPi;
    double lon = -kPi;
    for (int i = 0; i < 5; ++i) {
      p[1 + i] = sph2cart(lon, lat);
      lon = lon + dlon;
    }
    p[6] = {0, 0, -1};
    lat = -lat;
    lon = -(4.0 * kPi / 5.0);
    for (int i = 0; i < 5; ++i) {
      p[7 + i] = sph2cart(lon, lat);
      lon = lon + dlon;
    }
  }
  return p;
}

struct Tri {
  int a, b, c;
};

// Counter-clockwise neighbour rings from a closed, consistently oriented
// triangulation: in triangle (a,b,c), c follows b around a.
void build_rings(int n, const std::vector<Tri> &tris, std::vector<int> &nnb,
                 std::vector<int> &ring) {
  std::vector<int> cnt(n, 0);
  std::vector<std::array<int, 16>> from(n), to(n);
  auto add = [&](int v, int f, int t) {
    int k = cnt[v]++;
    if (k < 16) {
      from[v][k] = f;
      to[v][k] = t;
    }
  };
  for (const Tri &t : tris) {
    add(t.a, t.b, t.c);
    add(t.b, t.c, t.a);
    add(t.c, t.a, t.b);
  }
  nnb.assign(n, 0);
  ring.assign(static_cast<size_t>(n) * 6, -1);
  for (int v = 0; v < n; ++v) {
    int k = cnt[v];
    // start at the smallest-index neighbour
    int start = from[v][0];
    for (int i = 1; i < k; ++i) start = std::min(start, from[v][i]);
    int cur = start;
    for (int j = 0; j < k; ++j) {
      ring[static_cast<size_t>(v) * 6 + j] = cur;
      int nxt = -1;
      for (int i = 0; i < k; ++i)
        if (from[v][i] == cur) nxt = to[v][i];
      cur = nxt;
    }
    nnb[v] = k;
  }
}

struct Grid {
  int nv = 0, ne = 0, nt = 0;
  // 1-based index arrays, padded with 0
  std::vector<int32_t> nnb, v_nb, v_ed, v_tr, ttgout, tnrccw, hx_nr;
  std::vector<int32_t> ed_v, ed_sh, tr_v, tr_ed, tr_tg, tr_nr;
  std::vector<double> hx_areag, hxtr, trskw, v_p, v_lat, v_lon;
  std::vector<double> ed_leng, edhx_leng, ed_c, ed_c_lat, ed_c_lon, ed_tg, ed_nr;
  std::vector<double> edhx_c, edhx_nr, edhx_tg;
  std::vector<double> tr_areag, tr_trhx, tr_c, tr_c_lat;
  int64_t delaunay_bad = 0;
  double delaunay_margin = 0.0;
};

inline V3 getv(const std::vector<double> &a, size_t i) {
  return {a[3 * i], a[3 * i + 1], a[3 * i + 2]};
}
inline void setv(std::vector<double> &a, size_t i, const V3 &v) {
  a[3 * i] = v.x;
  a[3 * i + 1] = v.y;
  a[3 * i + 2] = v.z;
}

int build(Grid &g, int level, int pos) {
  // --- nodes and subdivision triangulation -----------------------------
  std::vector<V3> P = icosanodes0(pos);
  // level-0 faces: triples of mutually adjacent nodes (edge = min distance)
  std::vector<Tri> tris;
  {
    double dmin = 1e9;
    for (int i = 0; i < 12; ++i)
      for (int j = i + 1; j < 12; ++j) dmin = std::min(dmin, norm(sub(P[i], P[j])));
    auto adj = [&](int i, int j) { return norm(sub(P[i], P[j])) < dmin * (1.0 + 1e-6); };
    for (int i = 0; i < 12; ++i)
      for (int j = i + 1; j < 12; ++j)
        for (int k = j + 1; k < 12; ++k)
          if (adj(i, j) && adj(j, k) && adj(i, k)) {
            if (det3(P[i], P[j], P[k]) > 0)
              tris.push_back({i, j, k});
            else
              tris.push_back({i, k, j});
          }
    if (tris.size() != 20) return IMODEL_SWM_EINVAL;
  }
  std::vector<int> nnb, ring;
  for (int lev = 1; lev <= level; ++lev) {
    int n1 = static_cast<int>(P.size());
    build_rings(n1, tris, nnb, ring);
    // meshrefin (smeshpack.f90:1655-1671): new node for every edge i<k in
    // the order of i, then of i's neighbour list.
    std::vector<int> mid(static_cast<size_t>(n1) * 6, -1);
    P.reserve(static_cast<size_t>(4) * n1);
    for (int i = 0; i < n1; ++i) {
      for (int j = 0; j < nnb[i]; ++j) {
        int k = ring[static_cast<size_t>(i) * 6 + j];
        if (k > i) {
          V3 q = {0.5 * (P[i].x + P[k].x), 0.5 * (P[i].y + P[k].y), 0.5 * (P[i].z + P[k].z)};
          double r = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
          q = divs(q, r);
          mid[static_cast<size_t>(i) * 6 + j] = static_cast<int>(P.size());
          P.push_back(q);
        }
      }
    }
    auto midof = [&](int a, int b) -> int {
      int lo = std::min(a, b), hi = std::max(a, b);
      for (int j = 0; j < nnb[lo]; ++j)
        if (ring[static_cast<size_t>(lo) * 6 + j] == hi) return mid[static_cast<size_t>(lo) * 6 + j];
      return -1;
    };
    std::vector<Tri> nt;
    nt.reserve(tris.size() * 4);
    for (const Tri &t : tris) {
      int ab = midof(t.a, t.b), bc = midof(t.b, t.c), ca = midof(t.c, t.a);
      if (ab < 0 || bc < 0 || ca < 0) return IMODEL_SWM_EINVAL;
      nt.push_back({t.a, ab, ca});
      nt.push_back({ab, t.b, bc});
      nt.push_back({ca, bc, t.c});
      nt.push_back({ab, bc, ca});
    }
    tris.swap(nt);
  }
  const int nv = static_cast<int>(P.size());
  build_rings(nv, tris, nnb, ring);
  const int nt = 2 * nv - 4;
  const int ne = 3 * nv - 6;
  if (static_cast<int>(tris.size()) != nt) return IMODEL_SWM_EINVAL;
  g.nv = nv;
  g.ne = ne;
  g.nt = nt;

  // --- meshstruct (smeshpack.f90:370-1195), 0-based internally ----------
  std::vector<int> ved(static_cast<size_t>(nv) * 6, -1), vtr(static_cast<size_t>(nv) * 6, -1);
  g.v_p.resize(3 * static_cast<size_t>(nv));
  g.v_lat.resize(nv);
  g.v_lon.resize(nv);
  for (int i = 0; i < nv; ++i) {
    setv(g.v_p, i, P[i]);
    cart2sph(P[i].x, P[i].y, P[i].z, g.v_lon[i], g.v_lat[i]);
  }
  auto NB = [&](int i, int j) { return ring[static_cast<size_t>(i) * 6 + j]; };

  // edges (smeshpack.f90:706-752)
  std::vector<int> edv(2 * static_cast<size_t>(ne));
  g.ed_c.resize(3 * static_cast<size_t>(ne));
  g.ed_c_lat.resize(ne);
  g.ed_c_lon.resize(ne);
  g.ed_nr.resize(3 * static_cast<size_t>(ne));
  g.ed_tg.resize(3 * static_cast<size_t>(ne));
  g.ed_leng.resize(ne);
  {
    int l = 0;
    for (int i = 0; i < nv; ++i) {
      for (int j = 0; j < nnb[i]; ++j) {
        int k = NB(i, j);
        if (k > i) {
          if (l >= ne) return IMODEL_SWM_EINVAL;
          ved[static_cast<size_t>(i) * 6 + j] = l;
          edv[2 * static_cast<size_t>(l)] = i;
          edv[2 * static_cast<size_t>(l) + 1] = k;
          ++l;
        } else {
          for (int m = 0; m < nnb[k]; ++m)
            if (NB(k, m) == i) {
              ved[static_cast<size_t>(i) * 6 + j] = ved[static_cast<size_t>(k) * 6 + m];
              break;
            }
        }
      }
    }
    if (l != ne) return IMODEL_SWM_EINVAL;
  }
#pragma omp parallel for schedule(static)
  for (int l = 0; l < ne; ++l) {
    int i = edv[2 * static_cast<size_t>(l)], k = edv[2 * static_cast<size_t>(l) + 1];
    V3 c = midpoint(P[i], P[k]);
    setv(g.ed_c, l, c);
    cart2sph(c.x, c.y, c.z, g.ed_c_lon[l], g.ed_c_lat[l]);
    V3 nr = cross(P[i], P[k]);
    nr = divs(nr, norm(nr));
    V3 tg = cross(nr, c);
    tg = divs(tg, norm(tg));
    setv(g.ed_nr, l, nr);
    setv(g.ed_tg, l, tg);
    g.ed_leng[l] = arclen(P[i], P[k]);
  }
  auto getedge = [&](int a, int b) -> int {
    for (int j = 0; j < nnb[a]; ++j)
      if (NB(a, j) == b) return ved[static_cast<size_t>(a) * 6 + j];
    return -1;
  };

  // triangles (smeshpack.f90:779-862)
  std::vector<int> trv(3 * static_cast<size_t>(nt));
  {
    int k = 0;
    for (int i = 0; i < nv; ++i) {
      int nb = nnb[i];
      for (int j = 0; j < nb; ++j) {
        int ind[3] = {i, NB(i, j), NB(i, (j + 1) % nb)};
        int minind = std::min(ind[0], std::min(ind[1], ind[2]));
        if (minind == i) {
          if (k >= nt) return IMODEL_SWM_EINVAL;
          vtr[static_cast<size_t>(i) * 6 + j] = k;
          for (int q = 0; q < 3; ++q) trv[3 * static_cast<size_t>(k) + q] = ind[q];
          ++k;
        } else {
          int nm = nnb[minind];
          for (int l = 0; l < nm; ++l) {
            if (NB(minind, l) == i && minind == ind[2]) {
              vtr[static_cast<size_t>(i) * 6 + j] = vtr[static_cast<size_t>(minind) * 6 + l];
              break;
            }
            if (NB(minind, l) == i && minind == ind[1]) {
              int m = (l - 1 + nm) % nm;
              vtr[static_cast<size_t>(i) * 6 + j] = vtr[static_cast<size_t>(minind) * 6 + m];
              break;
            }
          }
        }
      }
    }
    if (k != nt) return IMODEL_SWM_EINVAL;
  }
  std::vector<int> tred(3 * static_cast<size_t>(nt)), edsh(2 * static_cast<size_t>(ne), -1);
  g.tr_tg.resize(3 * static_cast<size_t>(nt));
  g.tr_nr.resize(3 * static_cast<size_t>(nt));
  for (int k = 0; k < nt; ++k) {
    for (int l = 0; l < 3; ++l) {
      int m = (l + 1) % 3;
      int e = getedge(trv[3 * static_cast<size_t>(k) + l], trv[3 * static_cast<size_t>(k) + m]);
      if (e < 0) return IMODEL_SWM_EINVAL;
      tred[3 * static_cast<size_t>(k) + l] = e;
      if (edsh[2 * static_cast<size_t>(e)] < 0)
        edsh[2 * static_cast<size_t>(e)] = k;
      else
        edsh[2 * static_cast<size_t>(e) + 1] = k;
    }
  }
  int bad_sign = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad_sign)
  for (int k = 0; k < nt; ++k) {
    for (int l = 0; l < 3; ++l) {
      int m = (l + 1) % 3;
      int e = tred[3 * static_cast<size_t>(k) + l];
      V3 nr = cross(P[trv[3 * static_cast<size_t>(k) + l]], P[trv[3 * static_cast<size_t>(k) + m]]);
      nr = {-nr.x, -nr.y, -nr.z};
      nr = divs(nr, norm(nr));
      double dp = dot(nr, getv(g.ed_nr, e));
      if (std::fabs(std::fabs(dp) - 1.0) > kEps * 100.0) bad_sign += 1;
      if (dp > 0) {
        g.tr_nr[3 * static_cast<size_t>(k) + l] = 1;
        g.tr_tg[3 * static_cast<size_t>(k) + l] = -1;
      } else {
        g.tr_nr[3 * static_cast<size_t>(k) + l] = -1;
        g.tr_tg[3 * static_cast<size_t>(k) + l] = 1;
      }
    }
  }
  if (bad_sign) return IMODEL_SWM_EINVAL;

  // circumcentres and areas (smeshpack.f90:898-944)
  g.tr_c.resize(3 * static_cast<size_t>(nt));
  g.tr_c_lat.resize(nt);
  g.tr_areag.resize(nt);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nt; ++k) {
    V3 p1 = P[trv[3 * static_cast<size_t>(k)]], p2 = P[trv[3 * static_cast<size_t>(k) + 1]],
       p3 = P[trv[3 * static_cast<size_t>(k) + 2]];
    V3 c = trcircumc(p1, p2, p3);
    setv(g.tr_c, k, c);
    double lon;
    cart2sph(c.x, c.y, c.z, lon, g.tr_c_lat[k]);
    g.tr_areag[k] = sphtriarea(p1, p2, p3);
  }

  // Voronoi edges (smeshpack.f90:1016-1048)
  g.edhx_c.resize(3 * static_cast<size_t>(ne));
  g.edhx_nr.resize(3 * static_cast<size_t>(ne));
  g.edhx_tg.resize(3 * static_cast<size_t>(ne));
  g.edhx_leng.resize(ne);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < ne; ++i) {
    V3 c1 = getv(g.tr_c, edsh[2 * static_cast<size_t>(i)]);
    V3 c2 = getv(g.tr_c, edsh[2 * static_cast<size_t>(i) + 1]);
    V3 c = midpoint(c1, c2);
    setv(g.edhx_c, i, c);
    V3 nr = cross(c1, c2);
    nr = divs(nr, norm(nr));
    V3 tg = cross(nr, c);
    tg = divs(tg, norm(tg));
    setv(g.edhx_nr, i, nr);
    setv(g.edhx_tg, i, tg);
    g.edhx_leng[i] = arclen(c1, c2);
  }

  // Voronoi cells: signs and areas (smeshpack.f90:1071-1151, sphhxarea :4765)
  g.ttgout.assign(6 * static_cast<size_t>(nv), 0);
  g.tnrccw.assign(6 * static_cast<size_t>(nv), 0);
  g.hx_nr.assign(6 * static_cast<size_t>(nv), 0);
  g.hx_areag.resize(nv);
  int bad_hx = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad_hx)
  for (int i = 0; i < nv; ++i) {
    int nb = nnb[i];
    double area = 0.0;
    for (int j = 0; j < nb; ++j) {
      int j1 = vtr[static_cast<size_t>(i) * 6 + (j == 0 ? nb - 1 : j - 1)];
      int j2 = vtr[static_cast<size_t>(i) * 6 + j];
      int e = ved[static_cast<size_t>(i) * 6 + j];
      V3 cj1 = getv(g.tr_c, j1), cj2 = getv(g.tr_c, j2);
      V3 nr = cross(cj1, cj2);
      nr = {-nr.x, -nr.y, -nr.z};
      nr = divs(nr, norm(nr));
      double dp = dot(nr, getv(g.edhx_nr, e));
      if (std::fabs(std::fabs(dp) - 1.0) > kEps * 100.0) bad_hx += 1;
      int hnr = dp > 0 ? 1 : -1;
      int htg = -hnr;
      g.hx_nr[static_cast<size_t>(i) * 6 + j] = hnr;
      double d1 = dot(getv(g.ed_tg, e), muls(getv(g.edhx_nr, e), static_cast<double>(hnr)));
      g.ttgout[static_cast<size_t>(i) * 6 + j] = static_cast<int>(std::copysign(1.0, d1));
      double d2 = dot(getv(g.ed_nr, e), muls(getv(g.edhx_tg, e), static_cast<double>(htg)));
      g.tnrccw[static_cast<size_t>(i) * 6 + j] = static_cast<int>(std::copysign(1.0, d2));
      area = area + sphtriarea(P[i], cj1, cj2);
    }
    g.hx_areag[i] = area;
  }
  if (bad_hx) return IMODEL_SWM_EINVAL;

  // trhx_intersec_areas (smeshpack.f90:5080-5154)
  g.tr_trhx.resize(3 * static_cast<size_t>(nt));
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nt; ++k) {
    V3 pc = getv(g.tr_c, k);
    for (int j = 0; j < 3; ++j) {
      int ed1 = tred[3 * static_cast<size_t>(k) + (j == 0 ? 2 : j - 1)];
      int ed2 = tred[3 * static_cast<size_t>(k) + j];
      V3 ped1 = getv(g.ed_c, ed1), ped2 = getv(g.ed_c, ed2);
      V3 pv = P[trv[3 * static_cast<size_t>(k) + j]];
      double a1 = sphtriarea(pc, ped1, pv);
      if (det3(pc, ped1, pv) < 0) a1 = -a1;
      double a2 = sphtriarea(pc, pv, ped2);
      if (det3(pc, pv, ped2) < 0) a2 = -a2;
      g.tr_trhx[3 * static_cast<size_t>(k) + j] = a1 + a2;
    }
  }

  // hxtr_intersec_areas / areag and TRSK weights
  // (smeshpack.f90:4991-5078, interpack.f90:4016-4095)
  g.hxtr.assign(6 * static_cast<size_t>(nv), 0.0);
  g.trskw.assign(36 * static_cast<size_t>(nv), 0.0);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nv; ++c) {
    int n = nnb[c];
    V3 pc = P[c];
    double R[6];
    for (int j = 0; j < n; ++j) {
      int ed1 = ved[static_cast<size_t>(c) * 6 + j];
      int ed2 = ved[static_cast<size_t>(c) * 6 + (j + 1) % n];
      V3 ped1 = getv(g.edhx_c, ed1), ped2 = getv(g.edhx_c, ed2);
      V3 pv = getv(g.tr_c, vtr[static_cast<size_t>(c) * 6 + j]);
      double a1 = sphtriarea(pc, ped1, pv);
      if (det3(pc, ped1, pv) < 0) a1 = -a1;
      double a2 = sphtriarea(pc, pv, ped2);
      if (det3(pc, pv, ped2) < 0) a2 = -a2;
      double a = a1 + a2;
      R[j] = a / g.hx_areag[c];
      g.hxtr[static_cast<size_t>(c) * 6 + j] = R[j];
    }
    // trskw(i,j) stored at [c][j][i] (Fortran column-major per cell)
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) {
        double w;
        if (i == j) {
          w = 0.0;
        } else {
          double rsum = 0.0;
          if (j < i) {
            for (int k = i; k < n; ++k) rsum = rsum + R[k];
            for (int k = 0; k < j; ++k) rsum = rsum + R[k];
          } else {
            for (int k = i; k < j; ++k) rsum = rsum + R[k];
          }
          w = rsum - 0.5;
        }
        g.trskw[static_cast<size_t>(c) * 36 + static_cast<size_t>(j) * 6 + i] = w;
      }
    }
  }

  // Delaunay check: opposite vertex must not lie inside the circumcircle
  {
    int64_t bad = 0;
    double worst = -1e300;
#pragma omp parallel for schedule(static) reduction(+ : bad) reduction(max : worst)
    for (int e = 0; e < ne; ++e) {
      for (int s = 0; s < 2; ++s) {
        int t = edsh[2 * static_cast<size_t>(e) + s];
        int o = edsh[2 * static_cast<size_t>(e) + 1 - s];
        int a = trv[3 * static_cast<size_t>(t)], b = trv[3 * static_cast<size_t>(t) + 1],
            c = trv[3 * static_cast<size_t>(t) + 2];
        int d = -1;
        for (int q = 0; q < 3; ++q) {
          int x = trv[3 * static_cast<size_t>(o) + q];
          if (x != edv[2 * static_cast<size_t>(e)] && x != edv[2 * static_cast<size_t>(e) + 1]) d = x;
        }
        V3 nrm = cross(sub(P[b], P[a]), sub(P[c], P[a]));
        nrm = divs(nrm, norm(nrm));
        double m = dot(nrm, sub(P[d], P[a]));
        worst = std::max(worst, m);
        if (m > 1e-15) bad += 1;
      }
    }
    g.delaunay_bad = bad;
    g.delaunay_margin = -worst;
  }

  // --- export as 1-based reference arrays ------------------------------
  g.nnb.assign(nnb.begin(), nnb.end());
  g.v_nb.assign(6 * static_cast<size_t>(nv), 0);
  g.v_ed.assign(6 * static_cast<size_t>(nv), 0);
  g.v_tr.assign(6 * static_cast<size_t>(nv), 0);
  for (int i = 0; i < nv; ++i)
    for (int j = 0; j < nnb[i]; ++j) {
      size_t q = static_cast<size_t>(i) * 6 + j;
      g.v_nb[q] = ring[q] + 1;
      g.v_ed[q] = ved[q] + 1;
      g.v_tr[q] = vtr[q] + 1;
    }
  g.ed_v.resize(2 * static_cast<size_t>(ne));
  g.ed_sh.resize(2 * static_cast<size_t>(ne));
  for (size_t q = 0; q < 2 * static_cast<size_t>(ne); ++q) {
    g.ed_v[q] = edv[q] + 1;
    g.ed_sh[q] = edsh[q] + 1;
  }
  g.tr_v.resize(3 * static_cast<size_t>(nt));
  g.tr_ed.resize(3 * static_cast<size_t>(nt));
  for (size_t q = 0; q < 3 * static_cast<size_t>(nt); ++q) {
    g.tr_v[q] = trv[q] + 1;
    g.tr_ed[q] = tred[q] + 1;
  }
  return IMODEL_SWM_OK;
}

}  // namespace

extern "C" {

int imodel_mesh_build(int32_t level, int32_t pos, int32_t nthreads, void **grid) {
  if (!grid || level < 0 || level > 11 || (pos != 0 && pos != 1)) return IMODEL_SWM_EINVAL;
  *grid = nullptr;
#ifdef _OPENMP
  int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  Grid *g = new (std::nothrow) Grid();
  if (!g) return IMODEL_SWM_ENOMEM;
  int rc;
  try {
    rc = build(*g, level, pos);
  } catch (const std::bad_alloc &) {
    rc = IMODEL_SWM_ENOMEM;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  if (rc != IMODEL_SWM_OK) {
    delete g;
    return rc;
  }
  *grid = g;
  return IMODEL_SWM_OK;
}

int imodel_mesh_view(void *grid, imodel_swm_mesh *v) {
  if (!grid || !v) return IMODEL_SWM_EINVAL;
  Grid *g = static_cast<Grid *>(grid);
  std::memset(v, 0, sizeof(*v));
  v->nv = g->nv;
  v->ne = g->ne;
  v->nt = g->nt;
  v->nnb = g->nnb.data();
  v->v_nb = g->v_nb.data();
  v->v_ed = g->v_ed.data();
  v->v_tr = g->v_tr.data();
  v->hx_ttgout = g->ttgout.data();
  v->hx_tnrccw = g->tnrccw.data();
  v->hx_areag = g->hx_areag.data();
  v->hx_hxtr_area = g->hxtr.data();
  v->hx_trskw = g->trskw.data();
  v->v_p = g->v_p.data();
  v->v_lat = g->v_lat.data();
  v->ed_v = g->ed_v.data();
  v->ed_sh = g->ed_sh.data();
  v->ed_leng = g->ed_leng.data();
  v->edhx_leng = g->edhx_leng.data();
  v->ed_c = g->ed_c.data();
  v->ed_c_lat = g->ed_c_lat.data();
  v->ed_tg = g->ed_tg.data();
  v->ed_nr = g->ed_nr.data();
  v->tr_v = g->tr_v.data();
  v->tr_ed = g->tr_ed.data();
  v->tr_tg = g->tr_tg.data();
  v->tr_areag = g->tr_areag.data();
  v->tr_trhx_area = g->tr_trhx.data();
  v->tr_c_lat = g->tr_c_lat.data();
  v->erad = 6.37122e6;
  v->grav = 9.80616;
  v->omega = 7.292e-5;
  return IMODEL_SWM_OK;
}

int imodel_mesh_extra_view(void *grid, imodel_mesh_extra *v) {
  if (!grid || !v) return IMODEL_SWM_EINVAL;
  Grid *g = static_cast<Grid *>(grid);
  v->v_lon = g->v_lon.data();
  v->ed_c_lon = g->ed_c_lon.data();
  v->tr_c = g->tr_c.data();
  v->edhx_c = g->edhx_c.data();
  v->edhx_nr = g->edhx_nr.data();
  v->edhx_tg = g->edhx_tg.data();
  v->hx_nr = g->hx_nr.data();
  v->tr_nr = g->tr_nr.data();
  return IMODEL_SWM_OK;
}

int imodel_mesh_delaunay_violations(void *grid, int64_t *count, double *min_margin) {
  if (!grid) return IMODEL_SWM_EINVAL;
  Grid *g = static_cast<Grid *>(grid);
  if (count) *count = g->delaunay_bad;
  if (min_margin) *min_margin = g->delaunay_margin;
  return IMODEL_SWM_OK;
}

void imodel_mesh_free(void *grid) { delete static_cast<Grid *>(grid); }

}  // extern "C"
