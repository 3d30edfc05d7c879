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
// The Delaunay check at the end verifies the empty-circumcircle property on
// every edge.  Every loop runs on host threads (OpenMP); the numbering steps
// that the reference does in one serial sweep (new nodes, edges and
// triangles in the order of the lower node, then of its neighbour list) are
// a per-node count, a prefix sum and a fill, which gives the same numbers.
// The GPU back end (mesh_gpu.cu, imodel_mesh_build_gpu) runs the same
// construction as kernels, numbering included.

#include "imodel_mesh.h"
#include "mesh_internal.h"

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

using imodel::mesh::Grid;
using imodel::mesh::Topo;

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

// off[i + 1] = count(i), then the exclusive prefix sum: off[i] is the first
// number node i hands out when nodes number in index order.
template <class F>
void count_scan(int n, F count, std::vector<int> &off) {
  off.assign(static_cast<size_t>(n) + 1, 0);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) off[static_cast<size_t>(i) + 1] = count(i);
  for (int i = 0; i < n; ++i) off[static_cast<size_t>(i) + 1] += off[i];
}

// Counter-clockwise neighbour rings from a closed, consistently oriented
// triangulation: in triangle (a,b,c), c follows b around a.  Each ring
// starts at the node's smallest-index neighbour.  False if a node has more
// than six triangles (no icosahedral grid has).
bool build_rings(int n, const std::vector<Tri> &tris, std::vector<int> &nnb,
                 std::vector<int> &ring) {
  std::vector<int> cnt(n, 0), from(6 * static_cast<size_t>(n)), to(6 * static_cast<size_t>(n));
  const int64_t ntr = static_cast<int64_t>(tris.size());
  int over = 0;
#pragma omp parallel for schedule(static) reduction(+ : over)
  for (int64_t t = 0; t < ntr; ++t) {
    const Tri &T = tris[t];
    const int v[3] = {T.a, T.b, T.c}, f[3] = {T.b, T.c, T.a}, g[3] = {T.c, T.a, T.b};
    for (int q = 0; q < 3; ++q) {
      int k;
#pragma omp atomic capture
      k = cnt[v[q]]++;
      if (k < 6) {
        from[6 * static_cast<size_t>(v[q]) + k] = f[q];
        to[6 * static_cast<size_t>(v[q]) + k] = g[q];
      } else {
        ++over;
      }
    }
  }
  if (over) return false;
  nnb.assign(n, 0);
  ring.assign(static_cast<size_t>(n) * 6, -1);
#pragma omp parallel for schedule(static)
  for (int v = 0; v < n; ++v) {
    const int k = cnt[v];
    const int *fv = &from[6 * static_cast<size_t>(v)], *tv = &to[6 * static_cast<size_t>(v)];
    int start = fv[0];
    for (int i = 1; i < k; ++i) start = std::min(start, fv[i]);
    int cur = start;
    for (int j = 0; j < k; ++j) {
      ring[static_cast<size_t>(v) * 6 + j] = cur;
      int nxt = -1;
      for (int i = 0; i < k; ++i)
        if (fv[i] == cur) nxt = tv[i];
      cur = nxt;
    }
    nnb[v] = k;
  }
  return true;
}

template <class A>
inline V3 getv(const A &a, size_t i) {
  return {a[3 * i], a[3 * i + 1], a[3 * i + 2]};
}
template <class A>
inline void setv(A &a, size_t i, const V3 &v) {
  a[3 * i] = v.x;
  a[3 * i + 1] = v.y;
  a[3 * i + 2] = v.z;
}

// level-0 faces: triples of mutually adjacent nodes (edge = min distance),
// counter-clockwise seen from outside
bool level0_faces(const std::vector<V3> &P, std::vector<Tri> &tris) {
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
  return tris.size() == 20;
}

}  // namespace

namespace imodel {
namespace mesh {

int level0(int pos, std::vector<double> &p, std::vector<int> &tri) {
  const std::vector<V3> P = icosanodes0(pos);
  std::vector<Tri> tris;
  if (!level0_faces(P, tris)) return IMODEL_SWM_EINVAL;
  p.resize(36);
  for (int i = 0; i < 12; ++i) setv(p, i, P[i]);
  tri.resize(60);
  for (int t = 0; t < 20; ++t) {
    tri[3 * t] = tris[t].a;
    tri[3 * t + 1] = tris[t].b;
    tri[3 * t + 2] = tris[t].c;
  }
  return IMODEL_SWM_OK;
}

int topology(int level, int pos, Topo &T) {
  // --- nodes and subdivision triangulation -----------------------------
  std::vector<V3> P = icosanodes0(pos);
  std::vector<Tri> tris;
  if (!level0_faces(P, tris)) return IMODEL_SWM_EINVAL;
  std::vector<int> nnb, ring, off;
  auto NB = [&](int i, int j) { return ring[static_cast<size_t>(i) * 6 + j]; };
  for (int lev = 1; lev <= level; ++lev) {
    const int n1 = static_cast<int>(P.size());
    if (!build_rings(n1, tris, nnb, ring)) return IMODEL_SWM_EINVAL;
    // meshrefin (smeshpack.f90:1655-1671): a new node for every edge i < k
    // in the order of i, then of i's neighbour list
    count_scan(
        n1,
        [&](int i) {
          int c = 0;
          for (int j = 0; j < nnb[i]; ++j) c += NB(i, j) > i;
          return c;
        },
        off);
    std::vector<int> mid(static_cast<size_t>(n1) * 6, -1);
    P.resize(static_cast<size_t>(n1) + off[n1]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n1; ++i) {
      int q = n1 + off[i];
      for (int j = 0; j < nnb[i]; ++j) {
        const int k = NB(i, j);
        if (k > i) {
          V3 m = {0.5 * (P[i].x + P[k].x), 0.5 * (P[i].y + P[k].y), 0.5 * (P[i].z + P[k].z)};
          const double r = std::sqrt(m.x * m.x + m.y * m.y + m.z * m.z);
          P[q] = divs(m, r);
          mid[static_cast<size_t>(i) * 6 + j] = q;
          ++q;
        }
      }
    }
    auto midof = [&](int a, int b) -> int {
      const int lo = std::min(a, b), hi = std::max(a, b);
      for (int j = 0; j < nnb[lo]; ++j)
        if (NB(lo, j) == hi) return mid[static_cast<size_t>(lo) * 6 + j];
      return -1;
    };
    const int64_t ntr = static_cast<int64_t>(tris.size());
    std::vector<Tri> nt(4 * tris.size());
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t t = 0; t < ntr; ++t) {
      const Tri &o = tris[t];
      const int ab = midof(o.a, o.b), bc = midof(o.b, o.c), ca = midof(o.c, o.a);
      if (ab < 0 || bc < 0 || ca < 0) {
        ++bad;
        continue;
      }
      nt[4 * t] = {o.a, ab, ca};
      nt[4 * t + 1] = {ab, o.b, bc};
      nt[4 * t + 2] = {ca, bc, o.c};
      nt[4 * t + 3] = {ab, bc, ca};
    }
    if (bad) return IMODEL_SWM_EINVAL;
    tris.swap(nt);
  }
  const int nv = static_cast<int>(P.size());
  if (!build_rings(nv, tris, nnb, ring)) return IMODEL_SWM_EINVAL;
  const int nt = 2 * nv - 4;
  const int ne = 3 * nv - 6;
  if (static_cast<int>(tris.size()) != nt) return IMODEL_SWM_EINVAL;
  T.nv = nv;
  T.ne = ne;
  T.nt = nt;
  T.p.resize(3 * static_cast<size_t>(nv));
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) setv(T.p, i, P[i]);
  std::vector<V3>().swap(P);

  // --- meshstruct numbering (smeshpack.f90:706-862), 0-based -------------
  // edges: a new edge for every neighbour k > i, in the order of i, then of
  // i's neighbour list; edge (i, k) with k < i is the one k numbered
  std::vector<int> &ved = T.ved, &edv = T.edv;
  ved.assign(static_cast<size_t>(nv) * 6, -1);
  edv.assign(2 * static_cast<size_t>(ne), 0);
  count_scan(
      nv,
      [&](int i) {
        int c = 0;
        for (int j = 0; j < nnb[i]; ++j) c += NB(i, j) > i;
        return c;
      },
      off);
  if (off[nv] != ne) return IMODEL_SWM_EINVAL;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    int l = off[i];
    for (int j = 0; j < nnb[i]; ++j) {
      const int k = NB(i, j);
      if (k > i) {
        ved[static_cast<size_t>(i) * 6 + j] = l;
        edv[2 * static_cast<size_t>(l)] = i;
        edv[2 * static_cast<size_t>(l) + 1] = k;
        ++l;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    for (int j = 0; j < nnb[i]; ++j) {
      const int k = NB(i, j);
      if (k < i) {
        for (int m = 0; m < nnb[k]; ++m)
          if (NB(k, m) == i) {
            ved[static_cast<size_t>(i) * 6 + j] = ved[static_cast<size_t>(k) * 6 + m];
            break;
          }
      }
    }
  }
  // triangles (i, NB(i,j), NB(i,j+1)): numbered by their smallest node, in
  // the order of that node, then of its neighbour list; the others look
  // their number up at the smallest node
  std::vector<int> &vtr = T.vtr, &trv = T.trv;
  vtr.assign(static_cast<size_t>(nv) * 6, -1);
  trv.assign(3 * static_cast<size_t>(nt), 0);
  auto corner = [&](int i, int j, int q) {
    return q == 0 ? i : NB(i, (j + q - 1) % nnb[i]);
  };
  auto lowest = [&](int i, int j) {
    return std::min(i, std::min(corner(i, j, 1), corner(i, j, 2)));
  };
  count_scan(
      nv,
      [&](int i) {
        int c = 0;
        for (int j = 0; j < nnb[i]; ++j) c += lowest(i, j) == i;
        return c;
      },
      off);
  if (off[nv] != nt) return IMODEL_SWM_EINVAL;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    int k = off[i];
    for (int j = 0; j < nnb[i]; ++j)
      if (lowest(i, j) == i) {
        vtr[static_cast<size_t>(i) * 6 + j] = k;
        for (int q = 0; q < 3; ++q) trv[3 * static_cast<size_t>(k) + q] = corner(i, j, q);
        ++k;
      }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    for (int j = 0; j < nnb[i]; ++j) {
      const int minind = lowest(i, j);
      if (minind == i) continue;
      const int nm = nnb[minind];
      for (int l = 0; l < nm; ++l) {
        if (NB(minind, l) != i) continue;
        if (minind == corner(i, j, 2)) {
          vtr[static_cast<size_t>(i) * 6 + j] = vtr[static_cast<size_t>(minind) * 6 + l];
        } else {
          const int m = (l - 1 + nm) % nm;
          vtr[static_cast<size_t>(i) * 6 + j] = vtr[static_cast<size_t>(minind) * 6 + m];
        }
        break;
      }
    }
  }
  // edges of each triangle (edge l joins corners l and l+1) and the two
  // triangles of each edge, the lower number first (the order a sweep over
  // the triangles meets them)
  std::vector<int> &tred = T.tred, &edsh = T.edsh;
  tred.assign(3 * static_cast<size_t>(nt), -1);
  edsh.assign(2 * static_cast<size_t>(ne), -1);
  auto getedge = [&](int a, int b) -> int {
    for (int j = 0; j < nnb[a]; ++j)
      if (NB(a, j) == b) return ved[static_cast<size_t>(a) * 6 + j];
    return -1;
  };
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int k = 0; k < nt; ++k)
    for (int l = 0; l < 3; ++l) {
      const int e = getedge(trv[3 * static_cast<size_t>(k) + l],
                            trv[3 * static_cast<size_t>(k) + (l + 1) % 3]);
      if (e < 0) ++bad;
      tred[3 * static_cast<size_t>(k) + l] = e;
    }
  if (bad) return IMODEL_SWM_EINVAL;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int i = 0; i < nv; ++i) {
    const int nb = nnb[i];
    for (int j = 0; j < nb; ++j) {
      if (NB(i, j) < i) continue;
      const int e = ved[static_cast<size_t>(i) * 6 + j];
      const int a = vtr[static_cast<size_t>(i) * 6 + j];
      const int b = vtr[static_cast<size_t>(i) * 6 + (j - 1 + nb) % nb];
      if (e < 0 || a < 0 || b < 0 || a == b) {
        ++bad;
        continue;
      }
      edsh[2 * static_cast<size_t>(e)] = std::min(a, b);
      edsh[2 * static_cast<size_t>(e) + 1] = std::max(a, b);
    }
  }
  if (bad) return IMODEL_SWM_EINVAL;
  // every index the geometry gathers is in range (both back ends read
  // through them without further checks)
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int i = 0; i < nv; ++i) {
    if (nnb[i] < 3 || nnb[i] > 6) ++bad;
    for (int j = 0; j < nnb[i] && j < 6; ++j) {
      const size_t q = static_cast<size_t>(i) * 6 + j;
      if (ring[q] < 0 || ring[q] >= nv || ved[q] < 0 || ved[q] >= ne || vtr[q] < 0 || vtr[q] >= nt)
        ++bad;
    }
  }
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t q = 0; q < 2 * static_cast<int64_t>(ne); ++q)
    if (edv[q] < 0 || edv[q] >= nv || edsh[q] < 0 || edsh[q] >= nt) ++bad;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t q = 0; q < 3 * static_cast<int64_t>(nt); ++q)
    if (trv[q] < 0 || trv[q] >= nv || tred[q] < 0 || tred[q] >= ne) ++bad;
  if (bad) return IMODEL_SWM_EINVAL;
  T.nnb.swap(nnb);
  T.ring.swap(ring);
  return IMODEL_SWM_OK;
}

void export_topology(const Topo &T, Grid &g) {
  const int nv = T.nv, ne = T.ne, nt = T.nt;
  g.nv = nv;
  g.ne = ne;
  g.nt = nt;
  g.v_p.resize(T.p.size());
  g.nnb.resize(nv);
  g.v_nb.resize(6 * static_cast<size_t>(nv));
  g.v_ed.resize(6 * static_cast<size_t>(nv));
  g.v_tr.resize(6 * static_cast<size_t>(nv));
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    for (int c = 0; c < 3; ++c) g.v_p[3 * static_cast<size_t>(i) + c] = T.p[3 * static_cast<size_t>(i) + c];
    g.nnb[i] = T.nnb[i];
    for (int j = 0; j < 6; ++j) {
      const size_t q = static_cast<size_t>(i) * 6 + j;
      const bool on = j < T.nnb[i];
      g.v_nb[q] = on ? T.ring[q] + 1 : 0;
      g.v_ed[q] = on ? T.ved[q] + 1 : 0;
      g.v_tr[q] = on ? T.vtr[q] + 1 : 0;
    }
  }
  g.ed_v.resize(2 * static_cast<size_t>(ne));
  g.ed_sh.resize(2 * static_cast<size_t>(ne));
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < 2 * static_cast<int64_t>(ne); ++q) {
    g.ed_v[q] = T.edv[q] + 1;
    g.ed_sh[q] = T.edsh[q] + 1;
  }
  g.tr_v.resize(3 * static_cast<size_t>(nt));
  g.tr_ed.resize(3 * static_cast<size_t>(nt));
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < 3 * static_cast<int64_t>(nt); ++q) {
    g.tr_v[q] = T.trv[q] + 1;
    g.tr_ed[q] = T.tred[q] + 1;
  }
}

void touch(void *p, size_t bytes) {
  char *c = static_cast<char *>(p);
  const int64_t chunk = int64_t{1} << 20, n = static_cast<int64_t>((bytes + chunk - 1) / chunk);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    const size_t a = static_cast<size_t>(k) * chunk;
    std::memset(c + a, 0, std::min(static_cast<size_t>(chunk), bytes - a));
  }
}

}  // namespace mesh
}  // namespace imodel

namespace {

// meshstruct's geometry (smeshpack.f90:706-1151), the kite areas and the
// TRSK weights on host threads, entity by entity in the reference's
// arithmetic.  Returns an IMODEL_SWM_* status.
int geometry_host(const Topo &T, Grid &g) {
  const int nv = T.nv, ne = T.ne, nt = T.nt;
  const std::vector<int> &nnb = T.nnb, &ved = T.ved, &vtr = T.vtr, &edv = T.edv,
                         &edsh = T.edsh, &trv = T.trv, &tred = T.tred;
  auto P = [&](int i) { return getv(T.p, i); };
  g.v_lat.resize(nv);
  g.v_lon.resize(nv);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nv; ++i) {
    const V3 p = P(i);
    cart2sph(p.x, p.y, p.z, g.v_lon[i], g.v_lat[i]);
  }

  // edges (smeshpack.f90:706-752)
  g.ed_c.resize(3 * static_cast<size_t>(ne));
  g.ed_c_lat.resize(ne);
  g.ed_c_lon.resize(ne);
  g.ed_nr.resize(3 * static_cast<size_t>(ne));
  g.ed_tg.resize(3 * static_cast<size_t>(ne));
  g.ed_leng.resize(ne);
#pragma omp parallel for schedule(static)
  for (int l = 0; l < ne; ++l) {
    const V3 pi = P(edv[2 * static_cast<size_t>(l)]), pk = P(edv[2 * static_cast<size_t>(l) + 1]);
    V3 c = midpoint(pi, pk);
    setv(g.ed_c, l, c);
    cart2sph(c.x, c.y, c.z, g.ed_c_lon[l], g.ed_c_lat[l]);
    V3 nr = cross(pi, pk);
    nr = divs(nr, norm(nr));
    V3 tg = cross(nr, c);
    tg = divs(tg, norm(tg));
    setv(g.ed_nr, l, nr);
    setv(g.ed_tg, l, tg);
    g.ed_leng[l] = arclen(pi, pk);
  }

  // triangles: edge orientation signs (smeshpack.f90:779-862)
  g.tr_tg.resize(3 * static_cast<size_t>(nt));
  g.tr_nr.resize(3 * static_cast<size_t>(nt));
  int bad_sign = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad_sign)
  for (int k = 0; k < nt; ++k) {
    for (int l = 0; l < 3; ++l) {
      const int m = (l + 1) % 3;
      const int e = tred[3 * static_cast<size_t>(k) + l];
      V3 nr = cross(P(trv[3 * static_cast<size_t>(k) + l]), P(trv[3 * static_cast<size_t>(k) + m]));
      nr = {-nr.x, -nr.y, -nr.z};
      nr = divs(nr, norm(nr));
      const double dp = dot(nr, getv(g.ed_nr, e));
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
    const V3 p1 = P(trv[3 * static_cast<size_t>(k)]), p2 = P(trv[3 * static_cast<size_t>(k) + 1]),
             p3 = P(trv[3 * static_cast<size_t>(k) + 2]);
    const V3 c = trcircumc(p1, p2, p3);
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
    const V3 c1 = getv(g.tr_c, edsh[2 * static_cast<size_t>(i)]);
    const V3 c2 = getv(g.tr_c, edsh[2 * static_cast<size_t>(i) + 1]);
    const V3 c = midpoint(c1, c2);
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
    const int nb = nnb[i];
    double area = 0.0;
    for (int j = 0; j < nb; ++j) {
      const int j1 = vtr[static_cast<size_t>(i) * 6 + (j == 0 ? nb - 1 : j - 1)];
      const int j2 = vtr[static_cast<size_t>(i) * 6 + j];
      const int e = ved[static_cast<size_t>(i) * 6 + j];
      const V3 cj1 = getv(g.tr_c, j1), cj2 = getv(g.tr_c, j2);
      V3 nr = cross(cj1, cj2);
      nr = {-nr.x, -nr.y, -nr.z};
      nr = divs(nr, norm(nr));
      const double dp = dot(nr, getv(g.edhx_nr, e));
      if (std::fabs(std::fabs(dp) - 1.0) > kEps * 100.0) bad_hx += 1;
      const int hnr = dp > 0 ? 1 : -1;
      const int htg = -hnr;
      g.hx_nr[static_cast<size_t>(i) * 6 + j] = hnr;
      const double d1 = dot(getv(g.ed_tg, e), muls(getv(g.edhx_nr, e), static_cast<double>(hnr)));
      g.ttgout[static_cast<size_t>(i) * 6 + j] = static_cast<int>(std::copysign(1.0, d1));
      const double d2 = dot(getv(g.ed_nr, e), muls(getv(g.edhx_tg, e), static_cast<double>(htg)));
      g.tnrccw[static_cast<size_t>(i) * 6 + j] = static_cast<int>(std::copysign(1.0, d2));
      area = area + sphtriarea(P(i), cj1, cj2);
    }
    g.hx_areag[i] = area;
  }
  if (bad_hx) return IMODEL_SWM_EINVAL;

  // trhx_intersec_areas (smeshpack.f90:5080-5154)
  g.tr_trhx.resize(3 * static_cast<size_t>(nt));
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nt; ++k) {
    const V3 pc = getv(g.tr_c, k);
    for (int j = 0; j < 3; ++j) {
      const int ed1 = tred[3 * static_cast<size_t>(k) + (j == 0 ? 2 : j - 1)];
      const int ed2 = tred[3 * static_cast<size_t>(k) + j];
      const V3 ped1 = getv(g.ed_c, ed1), ped2 = getv(g.ed_c, ed2);
      const V3 pv = P(trv[3 * static_cast<size_t>(k) + j]);
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
    const int n = nnb[c];
    const V3 pc = P(c);
    double R[6];
    for (int j = 0; j < n; ++j) {
      const int ed1 = ved[static_cast<size_t>(c) * 6 + j];
      const int ed2 = ved[static_cast<size_t>(c) * 6 + (j + 1) % n];
      const V3 ped1 = getv(g.edhx_c, ed1), ped2 = getv(g.edhx_c, ed2);
      const V3 pv = getv(g.tr_c, vtr[static_cast<size_t>(c) * 6 + j]);
      double a1 = sphtriarea(pc, ped1, pv);
      if (det3(pc, ped1, pv) < 0) a1 = -a1;
      double a2 = sphtriarea(pc, pv, ped2);
      if (det3(pc, pv, ped2) < 0) a2 = -a2;
      const double a = a1 + a2;
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
        const int t = edsh[2 * static_cast<size_t>(e) + s];
        const int o = edsh[2 * static_cast<size_t>(e) + 1 - s];
        const int a = trv[3 * static_cast<size_t>(t)], b = trv[3 * static_cast<size_t>(t) + 1],
                  c = trv[3 * static_cast<size_t>(t) + 2];
        int d = -1;
        for (int q = 0; q < 3; ++q) {
          const int x = trv[3 * static_cast<size_t>(o) + q];
          if (x != edv[2 * static_cast<size_t>(e)] && x != edv[2 * static_cast<size_t>(e) + 1]) d = x;
        }
        if (d < 0) {  // the two triangles share all three nodes: not a grid
          bad += 1;
          continue;
        }
        V3 nrm = cross(sub(P(b), P(a)), sub(P(c), P(a)));
        nrm = divs(nrm, norm(nrm));
        const double m = dot(nrm, sub(P(d), P(a)));
        worst = std::max(worst, m);
        if (m > 1e-15) bad += 1;
      }
    }
    g.delaunay_bad = bad;
    g.delaunay_margin = -worst;
  }
  return IMODEL_SWM_OK;
}

// topology, the index arrays and one geometry back end into a new grid
template <class Geometry>
int build_grid(int32_t level, int32_t pos, void **grid, Geometry geometry) {
  if (!grid || level < 0 || level > 11 || (pos != 0 && pos != 1)) return IMODEL_SWM_EINVAL;
  *grid = nullptr;
  Grid *g = new (std::nothrow) Grid();
  if (!g) return IMODEL_SWM_ENOMEM;
  int rc;
  try {
    Topo t;
    rc = imodel::mesh::topology(level, pos, t);
    if (rc == IMODEL_SWM_OK) {
      imodel::mesh::export_topology(t, *g);
      rc = geometry(t, *g);
    }
  } catch (const std::bad_alloc &) {
    rc = IMODEL_SWM_ENOMEM;
  }
  if (rc != IMODEL_SWM_OK) {
    delete g;
    return rc;
  }
  *grid = g;
  return IMODEL_SWM_OK;
}

// the message of the last failed GPU build on this thread
thread_local const char *g_gpu_error = "";

}  // namespace

extern "C" {

int imodel_mesh_build(int32_t level, int32_t pos, int32_t nthreads, void **grid) {
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const int rc = build_grid(level, pos, grid, geometry_host);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(prev);
#endif
  return rc;
}

int imodel_mesh_build_gpu(int32_t level, int32_t pos, int32_t device, void **grid) {
  g_gpu_error = "";
  if (!grid || device < 0 || level < 0 || level > 11 || (pos != 0 && pos != 1))
    return IMODEL_SWM_EINVAL;
  *grid = nullptr;
  Grid *g = new (std::nothrow) Grid();
  if (!g) return IMODEL_SWM_ENOMEM;
  int rc;
  try {
    rc = imodel::mesh::build_gpu(level, pos, device, *g, &g_gpu_error);
  } catch (const std::bad_alloc &) {
    rc = IMODEL_SWM_ENOMEM;
  }
  if (rc != IMODEL_SWM_OK) {
    delete g;
    return rc;
  }
  *grid = g;
  return IMODEL_SWM_OK;
}

const char *imodel_mesh_gpu_last_error(void) { return g_gpu_error ? g_gpu_error : ""; }
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
