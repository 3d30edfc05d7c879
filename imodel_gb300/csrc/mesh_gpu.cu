// GPU back end of the grid builder: the subdivision and meshstruct's
// numbering (smeshpack.f90:1587-1675, :706-862) as per-node counts, prefix
// sums and fills, then meshstruct's per-entity geometry
// (smeshpack.f90:706-1151), the kite areas (trhx_intersec_areas
// :5080-5154, hxtr_intersec_areas :4991-5078), calc_trisk_weights
// (interpack.f90:3978-4098) and the Delaunay check, one thread per node,
// edge, triangle or cell.  geometry_gpu runs the geometry alone from a
// topology built on the host.
//
// Every value follows the host loops of mesh.cpp expression by expression,
// built with --fmad=false, so additions, products, quotients and square
// roots round as on the host.  The transcendental functions (atan, tan,
// atan2, asin) are CUDA's; they may differ from the host's C library in the
// last bit, so lengths, angles and areas agree with the host builder to a
// few units in the last place, and every index and sign array is identical.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "imodel_swm.h"
#include "mesh_internal.h"

namespace imodel {
namespace mesh {
namespace {

// constants.f90:31 and :45, as mesh.cpp forms them
__device__ const double kPi = 4.0 * static_cast<double>(0.78539816339744830961566f);
__device__ const double kEps = static_cast<double>(1.1920928955078125e-07f);

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 sub(const V3 &a, const V3 &b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
__device__ __forceinline__ double dot(const V3 &a, const V3 &b) {
  double s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
__device__ __forceinline__ V3 cross(const V3 &a, const V3 &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(const V3 &p) { return sqrt(dot(p, p)); }
__device__ __forceinline__ V3 divs(const V3 &p, double s) { return {p.x / s, p.y / s, p.z / s}; }
__device__ __forceinline__ V3 muls(const V3 &p, double s) { return {p.x * s, p.y * s, p.z * s}; }
__device__ __forceinline__ double det3(const V3 &a, const V3 &b, const V3 &c) {
  return dot(cross(a, b), c);
}
__device__ __forceinline__ V3 ld3(const double *a, int64_t i) {
  return {a[3 * i], a[3 * i + 1], a[3 * i + 2]};
}
__device__ __forceinline__ void st3(double *a, int64_t i, const V3 &v) {
  a[3 * i] = v.x;
  a[3 * i + 1] = v.y;
  a[3 * i + 2] = v.z;
}

// arclen, smeshpack.f90:4624-4657
__device__ double arclen(const V3 &p, const V3 &q) {
  const V3 s = {p.x + q.x, p.y + q.y, p.z + q.z};
  const double d = dot(s, s);
  if (d == 0.0) return kPi;
  if (d >= 4.0) return 0.0;
  return 2.0 * atan(sqrt((4.0 - d) / d));
}
// trcircumc, smeshpack.f90:4659-4687
__device__ V3 trcircumc(const V3 &p1, const V3 &p2, const V3 &p3) {
  const double tol = kEps / 100.0;
  if (norm(sub(p1, p2)) < tol || norm(sub(p2, p3)) < tol || norm(sub(p1, p3)) < tol)
    return {0.0, 0.0, 0.0};
  const V3 cp = cross(sub(p2, p1), sub(p3, p1));
  return divs(cp, norm(cp));
}
// sphtriarea (L'Huilier), smeshpack.f90:4710-4762
__device__ double sphtriarea(const V3 &p1, const V3 &p2, const V3 &p3) {
  const double tol = kEps / 100.0;
  if (norm(sub(p1, p2)) < tol || norm(sub(p2, p3)) < tol || norm(sub(p1, p3)) < tol)
    return 0.0;
  const double a = arclen(p1, p2);
  const double b = arclen(p2, p3);
  const double c = arclen(p3, p1);
  const double s = (a + b + c) / 2.0;
  double tmp = tan(s / 2.0) * tan((s - a) / 2.0);
  tmp = tmp * tan((s - b) / 2.0);
  tmp = tmp * tan((s - c) / 2.0);
  if (tmp < 0.0) return 0.0;
  return 4.0 * atan(sqrt(tmp));
}
// cart2sph, smeshpack.f90:4279-4313
__device__ void cart2sph(double x, double y, double z, double &lon, double &lat) {
  const double pnrm = sqrt(x * x + y * y + z * z);
  lon = (x != 0.0 || y != 0.0) ? atan2(y, x) : 0.0;
  lat = (pnrm != 0.0) ? asin(z / pnrm) : 0.0;
}
// midpoint_ed / midpoint_edhx, smeshpack.f90:6286-6334
__device__ V3 midpoint(const V3 &a, const V3 &b) {
  const V3 p = {(a.x + b.x) / 2.0, (a.y + b.y) / 2.0, (a.z + b.z) / 2.0};
  return divs(p, norm(p));
}

// device copies of the topology (0-based) and of the geometry being built
struct Dev {
  int nv, ne, nt;
  const double *p;
  const int *nnb, *ved, *vtr, *edv, *edsh, *trv, *tred;
  double *v_lat, *v_lon;
  double *ed_c, *ed_c_lat, *ed_c_lon, *ed_nr, *ed_tg, *ed_leng;
  int *tr_nr, *tr_tg;
  double *tr_c, *tr_c_lat, *tr_areag;
  double *edhx_c, *edhx_nr, *edhx_tg, *edhx_leng;
  int *hx_nr, *ttgout, *tnrccw;
  double *hx_areag, *tr_trhx, *hxtr, *trskw;
  double *worst;                // [blocks of k_delaunay]
  unsigned long long *counts;   // [0] bad signs, [1] bad cell signs, [2] Delaunay violations
};

constexpr int kThreads = 256;
inline int blocks(int64_t n) { return static_cast<int>((n + kThreads - 1) / kThreads); }

__global__ void k_nodes(Dev D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.nv) return;
  const V3 p = ld3(D.p, i);
  cart2sph(p.x, p.y, p.z, D.v_lon[i], D.v_lat[i]);
}

// edges (smeshpack.f90:706-752)
__global__ void k_edges(Dev D) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= D.ne) return;
  const V3 pi = ld3(D.p, D.edv[2 * l]), pk = ld3(D.p, D.edv[2 * l + 1]);
  const V3 c = midpoint(pi, pk);
  st3(D.ed_c, l, c);
  cart2sph(c.x, c.y, c.z, D.ed_c_lon[l], D.ed_c_lat[l]);
  V3 nr = cross(pi, pk);
  nr = divs(nr, norm(nr));
  V3 tg = cross(nr, c);
  tg = divs(tg, norm(tg));
  st3(D.ed_nr, l, nr);
  st3(D.ed_tg, l, tg);
  D.ed_leng[l] = arclen(pi, pk);
}

// triangles: edge orientation signs (smeshpack.f90:779-862), circumcentres
// and areas (:898-944)
__global__ void k_triangles(Dev D) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= D.nt) return;
  const int64_t k3 = 3 * static_cast<int64_t>(k);
  int bad = 0;
  for (int l = 0; l < 3; ++l) {
    const int m = (l + 1) % 3;
    const int e = D.tred[k3 + l];
    V3 nr = cross(ld3(D.p, D.trv[k3 + l]), ld3(D.p, D.trv[k3 + m]));
    nr = {-nr.x, -nr.y, -nr.z};
    nr = divs(nr, norm(nr));
    const double dp = dot(nr, ld3(D.ed_nr, e));
    if (fabs(fabs(dp) - 1.0) > kEps * 100.0) bad += 1;
    D.tr_nr[k3 + l] = dp > 0 ? 1 : -1;
    D.tr_tg[k3 + l] = dp > 0 ? -1 : 1;
  }
  if (bad) atomicAdd(&D.counts[0], static_cast<unsigned long long>(bad));
  const V3 p1 = ld3(D.p, D.trv[k3]), p2 = ld3(D.p, D.trv[k3 + 1]), p3 = ld3(D.p, D.trv[k3 + 2]);
  const V3 c = trcircumc(p1, p2, p3);
  st3(D.tr_c, k, c);
  double lon;
  cart2sph(c.x, c.y, c.z, lon, D.tr_c_lat[k]);
  D.tr_areag[k] = sphtriarea(p1, p2, p3);
}

// Voronoi edges (smeshpack.f90:1016-1048)
__global__ void k_voronoi_edges(Dev D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.ne) return;
  const V3 c1 = ld3(D.tr_c, D.edsh[2 * i]), c2 = ld3(D.tr_c, D.edsh[2 * i + 1]);
  const V3 c = midpoint(c1, c2);
  st3(D.edhx_c, i, c);
  V3 nr = cross(c1, c2);
  nr = divs(nr, norm(nr));
  V3 tg = cross(nr, c);
  tg = divs(tg, norm(tg));
  st3(D.edhx_nr, i, nr);
  st3(D.edhx_tg, i, tg);
  D.edhx_leng[i] = arclen(c1, c2);
}

// Voronoi cells: signs and areas (smeshpack.f90:1071-1151, sphhxarea :4765)
__global__ void k_cells(Dev D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.nv) return;
  const int64_t i6 = 6 * static_cast<int64_t>(i);
  const int nb = D.nnb[i];
  const V3 pi = ld3(D.p, i);
  double area = 0.0;
  int bad = 0;
  for (int j = 0; j < nb; ++j) {
    const int j1 = D.vtr[i6 + (j == 0 ? nb - 1 : j - 1)];
    const int j2 = D.vtr[i6 + j];
    const int e = D.ved[i6 + j];
    const V3 cj1 = ld3(D.tr_c, j1), cj2 = ld3(D.tr_c, j2);
    V3 nr = cross(cj1, cj2);
    nr = {-nr.x, -nr.y, -nr.z};
    nr = divs(nr, norm(nr));
    const double dp = dot(nr, ld3(D.edhx_nr, e));
    if (fabs(fabs(dp) - 1.0) > kEps * 100.0) bad += 1;
    const int hnr = dp > 0 ? 1 : -1;
    const int htg = -hnr;
    D.hx_nr[i6 + j] = hnr;
    const double d1 = dot(ld3(D.ed_tg, e), muls(ld3(D.edhx_nr, e), static_cast<double>(hnr)));
    D.ttgout[i6 + j] = static_cast<int>(copysign(1.0, d1));
    const double d2 = dot(ld3(D.ed_nr, e), muls(ld3(D.edhx_tg, e), static_cast<double>(htg)));
    D.tnrccw[i6 + j] = static_cast<int>(copysign(1.0, d2));
    area = area + sphtriarea(pi, cj1, cj2);
  }
  for (int j = nb; j < 6; ++j) D.hx_nr[i6 + j] = D.ttgout[i6 + j] = D.tnrccw[i6 + j] = 0;
  D.hx_areag[i] = area;
  if (bad) atomicAdd(&D.counts[1], static_cast<unsigned long long>(bad));
}

// trhx_intersec_areas (smeshpack.f90:5080-5154)
__global__ void k_trhx(Dev D) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= D.nt) return;
  const int64_t k3 = 3 * static_cast<int64_t>(k);
  const V3 pc = ld3(D.tr_c, k);
  for (int j = 0; j < 3; ++j) {
    const int ed1 = D.tred[k3 + (j == 0 ? 2 : j - 1)];
    const int ed2 = D.tred[k3 + j];
    const V3 ped1 = ld3(D.ed_c, ed1), ped2 = ld3(D.ed_c, ed2);
    const V3 pv = ld3(D.p, D.trv[k3 + j]);
    double a1 = sphtriarea(pc, ped1, pv);
    if (det3(pc, ped1, pv) < 0) a1 = -a1;
    double a2 = sphtriarea(pc, pv, ped2);
    if (det3(pc, pv, ped2) < 0) a2 = -a2;
    D.tr_trhx[k3 + j] = a1 + a2;
  }
}

// hxtr_intersec_areas / areag and the TRSK weights
// (smeshpack.f90:4991-5078, interpack.f90:4016-4095); trskw(i,j) of cell c
// at [c][j][i]
__global__ void k_kites(Dev D) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= D.nv) return;
  const int64_t c6 = 6 * static_cast<int64_t>(c);
  const int n = D.nnb[c];
  const V3 pc = ld3(D.p, c);
  const double area = D.hx_areag[c];
  double R[6];
  for (int j = 0; j < 6; ++j) {
    if (j >= n) {
      D.hxtr[c6 + j] = 0.0;
      continue;
    }
    const int ed1 = D.ved[c6 + j];
    const int ed2 = D.ved[c6 + (j + 1) % n];
    const V3 ped1 = ld3(D.edhx_c, ed1), ped2 = ld3(D.edhx_c, ed2);
    const V3 pv = ld3(D.tr_c, D.vtr[c6 + j]);
    double a1 = sphtriarea(pc, ped1, pv);
    if (det3(pc, ped1, pv) < 0) a1 = -a1;
    double a2 = sphtriarea(pc, pv, ped2);
    if (det3(pc, pv, ped2) < 0) a2 = -a2;
    const double a = a1 + a2;
    R[j] = a / area;
    D.hxtr[c6 + j] = R[j];
  }
  double *w = D.trskw + 36 * static_cast<int64_t>(c);
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) {
      double v = 0.0;
      if (i < n && j < n && i != j) {
        double rsum = 0.0;
        if (j < i) {
          for (int k = i; k < n; ++k) rsum = rsum + R[k];
          for (int k = 0; k < j; ++k) rsum = rsum + R[k];
        } else {
          for (int k = i; k < j; ++k) rsum = rsum + R[k];
        }
        v = rsum - 0.5;
      }
      w[6 * j + i] = v;
    }
}

// Delaunay check: the vertex opposite each edge must not lie inside the
// other triangle's circumcircle; per block the largest in-circle value
__global__ void k_delaunay(Dev D) {
  __shared__ double sw[kThreads];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double worst = -1e300;
  unsigned long long bad = 0;
  if (e < D.ne) {
    for (int s = 0; s < 2; ++s) {
      const int t = D.edsh[2 * e + s];
      const int o = D.edsh[2 * e + 1 - s];
      const int a = D.trv[3 * static_cast<int64_t>(t)], b = D.trv[3 * static_cast<int64_t>(t) + 1],
                c = D.trv[3 * static_cast<int64_t>(t) + 2];
      int d = -1;
      for (int q = 0; q < 3; ++q) {
        const int x = D.trv[3 * static_cast<int64_t>(o) + q];
        if (x != D.edv[2 * e] && x != D.edv[2 * e + 1]) d = x;
      }
      if (d < 0) {  // the two triangles share all three nodes: not a grid
        bad += 1;
        continue;
      }
      const V3 pa = ld3(D.p, a);
      V3 nrm = cross(sub(ld3(D.p, b), pa), sub(ld3(D.p, c), pa));
      nrm = divs(nrm, norm(nrm));
      const double m = dot(nrm, sub(ld3(D.p, d), pa));
      worst = fmax(worst, m);
      if (m > 1e-15) bad += 1;
    }
  }
  sw[threadIdx.x] = worst;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sw[threadIdx.x] = fmax(sw[threadIdx.x], sw[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) D.worst[blockIdx.x] = sw[0];
  if (bad) atomicAdd(&D.counts[2], bad);
}

// device buffers, freed in one place
struct Buffers {
  std::vector<void *> ptrs;
  cudaError_t err = cudaSuccess;
  template <class T>
  T *alloc(size_t n) {
    void *p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 16);
    if (err == cudaSuccess) ptrs.push_back(p);
    return static_cast<T *>(p);
  }
  template <class T>
  const T *upload(const std::vector<T> &v) {
    T *d = alloc<T>(v.size());
    if (err == cudaSuccess)
      err = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
  }
  template <class A, class T>
  void download(A &v, const T *d, size_t n) {
    v.resize(n);
    touch(v.data(), n * sizeof(T));  // map the pages on host threads first
    if (err == cudaSuccess) err = cudaMemcpy(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
  }
  ~Buffers() {
    for (void *p : ptrs) cudaFree(p);
  }
};

// ---- topology (mesh.cpp topology(), one kernel per loop) -----------------
// Per-node counts, an exclusive prefix sum and a fill hand out the numbers a
// serial sweep over the nodes (then over each node's neighbour list) would:
// the numbers mesh.cpp's host loops give.  Node positions are midpoints
// normalised with the host's operations in the host's order (no FMA), so
// they are bit-identical too.

struct Tri {
  int a, b, c;
};

// counts[3] of the topology kernels: [0] a node with more than six
// triangles, [1] a missing midpoint or edge, [2] an index out of range
struct TopoDev {
  int nv = 0;           // nodes of the current level
  double *p = nullptr;  // [nv_final][3]
  Tri *tri = nullptr, *tri2 = nullptr;  // [nt_final] each
  int *cnt = nullptr, *from = nullptr, *to = nullptr;  // [nv], [nv][6] x2
  int *nnb = nullptr, *ring = nullptr, *mid = nullptr;  // [nv], [nv][6] x2
  int *c = nullptr, *off = nullptr, *sums = nullptr;   // [nv], [nv + 1], scan blocks
  int *ved = nullptr, *vtr = nullptr, *edv = nullptr, *edsh = nullptr, *trv = nullptr,
      *tred = nullptr;
  unsigned long long *counts = nullptr;
};

// slot k of node v gets the (next, previous) pair of one of its triangles:
// in triangle (a, b, c), c follows b around a
__global__ void k_ring_pairs(int64_t ntr, const Tri *__restrict__ tri, int *cnt, int *from,
                             int *to, unsigned long long *counts) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= ntr) return;
  const Tri T = tri[t];
  const int v[3] = {T.a, T.b, T.c}, f[3] = {T.b, T.c, T.a}, g[3] = {T.c, T.a, T.b};
  for (int q = 0; q < 3; ++q) {
    const int k = atomicAdd(&cnt[v[q]], 1);
    if (k < 6) {
      from[6 * static_cast<int64_t>(v[q]) + k] = f[q];
      to[6 * static_cast<int64_t>(v[q]) + k] = g[q];
    } else {
      atomicAdd(&counts[0], 1ull);
    }
  }
}

// the counter-clockwise ring of node v from its pairs, starting at its
// smallest-index neighbour (build_rings in mesh.cpp); a walk that breaks
// (not a closed, consistently oriented triangulation) is counted
__global__ void k_rings(int n, const int *__restrict__ cnt, const int *__restrict__ from,
                        const int *__restrict__ to, int *nnb, int *ring,
                        unsigned long long *counts) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const int k = min(cnt[v], 6);
  const int *fv = from + 6 * static_cast<int64_t>(v), *tv = to + 6 * static_cast<int64_t>(v);
  int *rv = ring + 6 * static_cast<int64_t>(v);
  int cur = k > 0 ? fv[0] : -1;
  for (int i = 1; i < k; ++i) cur = min(cur, fv[i]);
  bool broken = k < 3;
  for (int j = 0; j < 6; ++j) {
    if (j < k && (cur < 0 || cur >= n)) broken = true;
    rv[j] = j < k ? cur : -1;
    int nxt = -1;
    for (int i = 0; i < k; ++i)
      if (fv[i] == cur) nxt = tv[i];
    cur = nxt;
  }
  nnb[v] = k;
  if (broken) atomicAdd(&counts[1], 1ull);
}

// c[i] = how many numbers node i hands out: neighbours above it (edges,
// midpoints) or triangles whose smallest corner it is
__device__ __forceinline__ int tri_corner(const int *ring, const int *nnb, int i, int j, int q) {
  return q == 0 ? i : ring[6 * static_cast<int64_t>(i) + (j + q - 1) % nnb[i]];
}
__device__ __forceinline__ int tri_lowest(const int *ring, const int *nnb, int i, int j) {
  return min(i, min(tri_corner(ring, nnb, i, j, 1), tri_corner(ring, nnb, i, j, 2)));
}
__global__ void k_count(int n, const int *__restrict__ nnb, const int *__restrict__ ring,
                        int triangles, int *c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k = 0;
  for (int j = 0; j < nnb[i]; ++j)
    k += triangles ? tri_lowest(ring, nnb, i, j) == i : ring[6 * static_cast<int64_t>(i) + j] > i;
  c[i] = k;
}

// exclusive prefix sum off[0..n] of c[0..n): kScanChunk values per block,
// kScanItems consecutive values per thread
constexpr int kScanItems = 8;
constexpr int kScanChunk = kThreads * kScanItems;

// exclusive scan of x over the block; *total receives the block's sum
__device__ int block_scan(int x, int *total) {
  __shared__ int warp_sums[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = x;
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    int s = lane < kThreads / 32 ? warp_sums[lane] : 0;
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    if (lane < kThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const int base = w > 0 ? warp_sums[w - 1] : 0;
  *total = warp_sums[kThreads / 32 - 1];
  __syncthreads();
  return base + inc - x;
}

__global__ void k_scan_sums(int n, const int *__restrict__ c, int *sums) {
  const int64_t b0 = static_cast<int64_t>(blockIdx.x) * kScanChunk + threadIdx.x * kScanItems;
  int x = 0;
  for (int q = 0; q < kScanItems; ++q)
    if (b0 + q < n) x += c[b0 + q];
  int total;
  block_scan(x, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: exclusive scan of the nb block sums in place
__global__ void k_scan_tops(int nb, int *sums) {
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += kThreads) {
    const int b = b0 + threadIdx.x;
    const int x = b < nb ? sums[b] : 0;
    int total;
    const int ex = block_scan(x, &total);
    if (b < nb) sums[b] = carry + ex;
    carry += total;
  }
}

__global__ void k_scan_fill(int n, const int *__restrict__ c, const int *__restrict__ sums,
                            int *off) {
  const int64_t b0 = static_cast<int64_t>(blockIdx.x) * kScanChunk + threadIdx.x * kScanItems;
  int v[kScanItems];
  int x = 0;
  for (int q = 0; q < kScanItems; ++q) {
    v[q] = b0 + q < n ? c[b0 + q] : 0;
    x += v[q];
  }
  int total;
  int run = sums[blockIdx.x] + block_scan(x, &total);
  if (blockIdx.x == 0 && threadIdx.x == 0) off[0] = 0;
  for (int q = 0; q < kScanItems; ++q) {
    run += v[q];
    if (b0 + q < n) off[b0 + q + 1] = run;
  }
}

// meshrefin (smeshpack.f90:1655-1671): a new node at the normalised
// midpoint of every edge i < k, numbered in the order of i, then of i's
// neighbour list; mid[i][j] its number (-1 for j's neighbour below i)
__global__ void k_midpoints(int n1, const int *__restrict__ nnb, const int *__restrict__ ring,
                            const int *__restrict__ off, double *p, int *mid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n1) return;
  int q = n1 + off[i];
  const V3 pi = ld3(p, i);
  for (int j = 0; j < 6; ++j) {
    const int k = j < nnb[i] ? ring[6 * static_cast<int64_t>(i) + j] : -1;
    int m = -1;
    if (k > i) {
      const V3 pk = ld3(p, k);
      const V3 c = {0.5 * (pi.x + pk.x), 0.5 * (pi.y + pk.y), 0.5 * (pi.z + pk.z)};
      const double r = sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
      st3(p, q, divs(c, r));
      m = q++;
    }
    mid[6 * static_cast<int64_t>(i) + j] = m;
  }
}

// the 4-way subdivision of every triangle; a missing midpoint (not a closed
// triangulation) leaves the four children at node 0 and is counted
__global__ void k_subdivide(int64_t ntr, const Tri *__restrict__ tri, const int *__restrict__ nnb,
                            const int *__restrict__ ring, const int *__restrict__ mid, Tri *out,
                            unsigned long long *counts) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= ntr) return;
  const Tri o = tri[t];
  auto midof = [&](int a, int b) {
    const int lo = min(a, b), hi = max(a, b);
    for (int j = 0; j < nnb[lo]; ++j)
      if (ring[6 * static_cast<int64_t>(lo) + j] == hi) return mid[6 * static_cast<int64_t>(lo) + j];
    return -1;
  };
  const int ab = midof(o.a, o.b), bc = midof(o.b, o.c), ca = midof(o.c, o.a);
  if (ab < 0 || bc < 0 || ca < 0) {
    atomicAdd(&counts[1], 1ull);
    for (int q = 0; q < 4; ++q) out[4 * t + q] = {0, 0, 0};
    return;
  }
  out[4 * t] = {o.a, ab, ca};
  out[4 * t + 1] = {ab, o.b, bc};
  out[4 * t + 2] = {ca, bc, o.c};
  out[4 * t + 3] = {ab, bc, ca};
}

// edges (smeshpack.f90:706-752 numbering): a new edge for every neighbour
// k > i, in the order of i, then of i's neighbour list
__global__ void k_edge_numbers(int nv, const int *__restrict__ nnb, const int *__restrict__ ring,
                               const int *__restrict__ off, int *ved, int *edv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int l = off[i];
  for (int j = 0; j < 6; ++j) {
    const int k = j < nnb[i] ? ring[6 * static_cast<int64_t>(i) + j] : -1;
    int e = -1;
    if (k > i) {
      edv[2 * static_cast<int64_t>(l)] = i;
      edv[2 * static_cast<int64_t>(l) + 1] = k;
      e = l++;
    }
    ved[6 * static_cast<int64_t>(i) + j] = e;
  }
}

// edge (i, k) with k < i is the one k numbered
__global__ void k_edge_lookup(int nv, const int *__restrict__ nnb, const int *__restrict__ ring,
                              int *ved) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  for (int j = 0; j < nnb[i]; ++j) {
    const int k = ring[6 * static_cast<int64_t>(i) + j];
    if (k < 0 || k >= i) continue;
    for (int m = 0; m < nnb[k]; ++m)
      if (ring[6 * static_cast<int64_t>(k) + m] == i) {
        ved[6 * static_cast<int64_t>(i) + j] = ved[6 * static_cast<int64_t>(k) + m];
        break;
      }
  }
}

// triangles (i, NB(i,j), NB(i,j+1)): numbered by their smallest node, in
// the order of that node, then of its neighbour list
__global__ void k_tri_numbers(int nv, const int *__restrict__ nnb, const int *__restrict__ ring,
                              const int *__restrict__ off, int *vtr, int *trv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  int k = off[i];
  for (int j = 0; j < 6; ++j) {
    int t = -1;
    if (j < nnb[i] && tri_lowest(ring, nnb, i, j) == i) {
      for (int q = 0; q < 3; ++q) trv[3 * static_cast<int64_t>(k) + q] = tri_corner(ring, nnb, i, j, q);
      t = k++;
    }
    vtr[6 * static_cast<int64_t>(i) + j] = t;
  }
}

// the other corners look the number up at the smallest node
__global__ void k_tri_lookup(int nv, const int *__restrict__ nnb, const int *__restrict__ ring,
                             int *vtr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  for (int j = 0; j < nnb[i]; ++j) {
    const int minind = tri_lowest(ring, nnb, i, j);
    if (minind == i || minind < 0) continue;
    const int nm = nnb[minind];
    for (int l = 0; l < nm; ++l) {
      if (ring[6 * static_cast<int64_t>(minind) + l] != i) continue;
      const int m = minind == tri_corner(ring, nnb, i, j, 2) ? l : (l - 1 + nm) % nm;
      vtr[6 * static_cast<int64_t>(i) + j] = vtr[6 * static_cast<int64_t>(minind) + m];
      break;
    }
  }
}

// edges of each triangle (edge l joins corners l and l+1)
__global__ void k_tri_edges(int nt, const int *__restrict__ nnb, const int *__restrict__ ring,
                            const int *__restrict__ ved, const int *__restrict__ trv, int *tred,
                            unsigned long long *counts) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  for (int l = 0; l < 3; ++l) {
    const int a = trv[3 * static_cast<int64_t>(k) + l], b = trv[3 * static_cast<int64_t>(k) + (l + 1) % 3];
    int e = -1;
    for (int j = 0; j < nnb[a]; ++j)
      if (ring[6 * static_cast<int64_t>(a) + j] == b) e = ved[6 * static_cast<int64_t>(a) + j];
    if (e < 0) atomicAdd(&counts[1], 1ull);
    tred[3 * static_cast<int64_t>(k) + l] = e;
  }
}

// the two triangles of each edge, the lower number first
__global__ void k_edge_tris(int nv, const int *__restrict__ nnb, const int *__restrict__ ring,
                            const int *__restrict__ ved, const int *__restrict__ vtr, int *edsh,
                            unsigned long long *counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int nb = nnb[i];
  for (int j = 0; j < nb; ++j) {
    if (ring[6 * static_cast<int64_t>(i) + j] < i) continue;
    const int e = ved[6 * static_cast<int64_t>(i) + j];
    const int a = vtr[6 * static_cast<int64_t>(i) + j];
    const int b = vtr[6 * static_cast<int64_t>(i) + (j - 1 + nb) % nb];
    if (e < 0 || a < 0 || b < 0 || a == b) {
      atomicAdd(&counts[1], 1ull);
      continue;
    }
    edsh[2 * static_cast<int64_t>(e)] = min(a, b);
    edsh[2 * static_cast<int64_t>(e) + 1] = max(a, b);
  }
}

// every index the geometry gathers is in range (blocks [0, bv) the nodes,
// [bv, bv + be) the edge entries, the rest the triangle entries)
__global__ void k_range_check(int nv, int ne, int nt, int bv, int be, const int *__restrict__ nnb,
                              const int *__restrict__ ring, const int *__restrict__ ved,
                              const int *__restrict__ vtr, const int *__restrict__ edv,
                              const int *__restrict__ edsh, const int *__restrict__ trv,
                              const int *__restrict__ tred, unsigned long long *counts) {
  int bad = 0;
  if (static_cast<int>(blockIdx.x) < bv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) {
      if (nnb[i] < 3 || nnb[i] > 6) ++bad;
      for (int j = 0; j < nnb[i] && j < 6; ++j) {
        const int64_t q = 6 * static_cast<int64_t>(i) + j;
        if (ring[q] < 0 || ring[q] >= nv || ved[q] < 0 || ved[q] >= ne || vtr[q] < 0 || vtr[q] >= nt)
          ++bad;
      }
    }
  } else if (static_cast<int>(blockIdx.x) < bv + be) {
    const int64_t q = (blockIdx.x - bv) * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (q < 2 * static_cast<int64_t>(ne) &&
        (edv[q] < 0 || edv[q] >= nv || edsh[q] < 0 || edsh[q] >= nt))
      ++bad;
  } else {
    const int64_t q = (blockIdx.x - bv - be) * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (q < 3 * static_cast<int64_t>(nt) &&
        (trv[q] < 0 || trv[q] >= nv || tred[q] < 0 || tred[q] >= ne))
      ++bad;
  }
  if (bad) atomicAdd(&counts[2], static_cast<unsigned long long>(bad));
}

// the grid's 1-based index arrays, 0-padded (export_topology in mesh.cpp)
__global__ void k_export(int nv, int ne, int nt, int bv, int be, const int *__restrict__ nnb,
                         const int *__restrict__ ring, const int *__restrict__ ved,
                         const int *__restrict__ vtr, const int *__restrict__ edv,
                         const int *__restrict__ edsh, const int *__restrict__ trv,
                         const int *__restrict__ tred, int *v_nb, int *v_ed, int *v_tr, int *ed_v,
                         int *ed_sh, int *tr_v, int *tr_ed) {
  if (static_cast<int>(blockIdx.x) < bv) {
    const int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (q >= 6 * static_cast<int64_t>(nv)) return;
    const bool on = q % 6 < nnb[q / 6];
    v_nb[q] = on ? ring[q] + 1 : 0;
    v_ed[q] = on ? ved[q] + 1 : 0;
    v_tr[q] = on ? vtr[q] + 1 : 0;
  } else if (static_cast<int>(blockIdx.x) < bv + be) {
    const int64_t q = (blockIdx.x - bv) * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (q >= 2 * static_cast<int64_t>(ne)) return;
    ed_v[q] = edv[q] + 1;
    ed_sh[q] = edsh[q] + 1;
  } else {
    const int64_t q = (blockIdx.x - bv - be) * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (q >= 3 * static_cast<int64_t>(nt)) return;
    tr_v[q] = trv[q] + 1;
    tr_ed[q] = tred[q] + 1;
  }
}

// c -> off over n nodes; *total receives off[n]
cudaError_t scan(const TopoDev &T, int n, int *total) {
  const int nb = static_cast<int>((static_cast<int64_t>(n) + kScanChunk - 1) / kScanChunk);
  k_scan_sums<<<nb, kThreads>>>(n, T.c, T.sums);
  k_scan_tops<<<1, kThreads>>>(nb, T.sums);
  k_scan_fill<<<nb, kThreads>>>(n, T.c, T.sums, T.off);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(total, T.off + n, sizeof(int), cudaMemcpyDeviceToHost);
  return e;
}

// rings of the first n nodes from ntr triangles; false if a node has more
// than six triangles
cudaError_t rings(const TopoDev &T, int n, int64_t ntr, const Tri *tri, bool *ok) {
  cudaError_t e = cudaMemset(T.cnt, 0, static_cast<size_t>(n) * sizeof(int));
  if (e != cudaSuccess) return e;
  k_ring_pairs<<<blocks(ntr), kThreads>>>(ntr, tri, T.cnt, T.from, T.to, T.counts);
  k_rings<<<blocks(n), kThreads>>>(n, T.cnt, T.from, T.to, T.nnb, T.ring, T.counts);
  e = cudaGetLastError();
  unsigned long long c[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(c, T.counts, sizeof(c), cudaMemcpyDeviceToHost);
  *ok = c[0] == 0 && c[1] == 0;
  return e;
}

}  // namespace

namespace {

int cuda_status(cudaError_t e) {
  return e == cudaErrorMemoryAllocation ? IMODEL_SWM_ENOMEM : IMODEL_SWM_ECUDA;
}

// the geometry kernels and the downloads into g, D's topology (0-based)
// already on the device
int geometry_dev(Buffers &B, Dev &D, Grid &g, const char **why) {
  const int nv = D.nv, ne = D.ne, nt = D.nt;
  const size_t v6 = 6 * static_cast<size_t>(nv), e3 = 3 * static_cast<size_t>(ne),
               t3 = 3 * static_cast<size_t>(nt);
  D.v_lat = B.alloc<double>(nv);
  D.v_lon = B.alloc<double>(nv);
  D.ed_c = B.alloc<double>(e3);
  D.ed_c_lat = B.alloc<double>(ne);
  D.ed_c_lon = B.alloc<double>(ne);
  D.ed_nr = B.alloc<double>(e3);
  D.ed_tg = B.alloc<double>(e3);
  D.ed_leng = B.alloc<double>(ne);
  D.tr_nr = B.alloc<int>(t3);
  D.tr_tg = B.alloc<int>(t3);
  D.tr_c = B.alloc<double>(t3);
  D.tr_c_lat = B.alloc<double>(nt);
  D.tr_areag = B.alloc<double>(nt);
  D.edhx_c = B.alloc<double>(e3);
  D.edhx_nr = B.alloc<double>(e3);
  D.edhx_tg = B.alloc<double>(e3);
  D.edhx_leng = B.alloc<double>(ne);
  D.hx_nr = B.alloc<int>(v6);
  D.ttgout = B.alloc<int>(v6);
  D.tnrccw = B.alloc<int>(v6);
  D.hx_areag = B.alloc<double>(nv);
  D.tr_trhx = B.alloc<double>(t3);
  D.hxtr = B.alloc<double>(v6);
  D.trskw = B.alloc<double>(36 * static_cast<size_t>(nv));
  const int nbd = blocks(ne);
  D.worst = B.alloc<double>(nbd);
  D.counts = B.alloc<unsigned long long>(3);
  if (B.err == cudaSuccess) B.err = cudaMemset(D.counts, 0, 3 * sizeof(unsigned long long));
  if (B.err != cudaSuccess) {
    *why = cudaGetErrorString(B.err);
    return B.err == cudaErrorMemoryAllocation ? IMODEL_SWM_ENOMEM : IMODEL_SWM_ECUDA;
  }
  // each kernel reads only what the ones before it wrote
  k_nodes<<<blocks(nv), kThreads>>>(D);
  k_edges<<<blocks(ne), kThreads>>>(D);
  k_triangles<<<blocks(nt), kThreads>>>(D);
  k_voronoi_edges<<<blocks(ne), kThreads>>>(D);
  k_cells<<<blocks(nv), kThreads>>>(D);
  k_trhx<<<blocks(nt), kThreads>>>(D);
  k_kites<<<blocks(nv), kThreads>>>(D);
  k_delaunay<<<nbd, kThreads>>>(D);
  B.err = cudaGetLastError();
  if (B.err == cudaSuccess) B.err = cudaDeviceSynchronize();
  unsigned long long counts[3] = {0, 0, 0};
  if (B.err == cudaSuccess)
    B.err = cudaMemcpy(counts, D.counts, sizeof(counts), cudaMemcpyDeviceToHost);
  if (B.err == cudaSuccess && (counts[0] || counts[1])) return IMODEL_SWM_EINVAL;
  std::vector<double> worst;
  B.download(worst, D.worst, nbd);
  B.download(g.v_lat, D.v_lat, nv);
  B.download(g.v_lon, D.v_lon, nv);
  B.download(g.ed_c, D.ed_c, e3);
  B.download(g.ed_c_lat, D.ed_c_lat, ne);
  B.download(g.ed_c_lon, D.ed_c_lon, ne);
  B.download(g.ed_nr, D.ed_nr, e3);
  B.download(g.ed_tg, D.ed_tg, e3);
  B.download(g.ed_leng, D.ed_leng, ne);
  B.download(g.tr_nr, D.tr_nr, t3);
  B.download(g.tr_tg, D.tr_tg, t3);
  B.download(g.tr_c, D.tr_c, t3);
  B.download(g.tr_c_lat, D.tr_c_lat, nt);
  B.download(g.tr_areag, D.tr_areag, nt);
  B.download(g.edhx_c, D.edhx_c, e3);
  B.download(g.edhx_nr, D.edhx_nr, e3);
  B.download(g.edhx_tg, D.edhx_tg, e3);
  B.download(g.edhx_leng, D.edhx_leng, ne);
  B.download(g.hx_nr, D.hx_nr, v6);
  B.download(g.ttgout, D.ttgout, v6);
  B.download(g.tnrccw, D.tnrccw, v6);
  B.download(g.hx_areag, D.hx_areag, nv);
  B.download(g.tr_trhx, D.tr_trhx, t3);
  B.download(g.hxtr, D.hxtr, v6);
  B.download(g.trskw, D.trskw, 36 * static_cast<size_t>(nv));
  if (B.err != cudaSuccess) {
    *why = cudaGetErrorString(B.err);
    return IMODEL_SWM_ECUDA;
  }
  double w = -1e300;
  for (double x : worst) w = x > w ? x : w;
  g.delaunay_bad = static_cast<int64_t>(counts[2]);
  g.delaunay_margin = -w;
  return IMODEL_SWM_OK;
}

}  // namespace

int geometry_gpu(const Topo &T, Grid &g, int device, const char **why) {
  *why = "";
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return IMODEL_SWM_ECUDA;
  }
  Buffers B;
  Dev D;
  D.nv = T.nv;
  D.ne = T.ne;
  D.nt = T.nt;
  D.p = B.upload(T.p);
  D.nnb = B.upload(T.nnb);
  D.ved = B.upload(T.ved);
  D.vtr = B.upload(T.vtr);
  D.edv = B.upload(T.edv);
  D.edsh = B.upload(T.edsh);
  D.trv = B.upload(T.trv);
  D.tred = B.upload(T.tred);
  return geometry_dev(B, D, g, why);
}

int build_gpu(int level, int pos, int device, Grid &g, const char **why) {
  *why = "";
  std::vector<double> p0;
  std::vector<int> t0;
  int rc = level0(pos, p0, t0);
  if (rc) return rc;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return IMODEL_SWM_ECUDA;
  }
  const int64_t f = int64_t{1} << (2 * level);  // 4^level
  const int nv = static_cast<int>(10 * f + 2), ne = static_cast<int>(30 * f),
            nt = static_cast<int>(20 * f);
  const size_t v6 = 6 * static_cast<size_t>(nv);
  Buffers B;
  TopoDev T;
  T.p = B.alloc<double>(3 * static_cast<size_t>(nv));
  T.tri = B.alloc<Tri>(nt);
  T.tri2 = B.alloc<Tri>(nt);
  T.cnt = B.alloc<int>(nv);
  T.from = B.alloc<int>(v6);
  T.to = B.alloc<int>(v6);
  T.nnb = B.alloc<int>(nv);
  T.ring = B.alloc<int>(v6);
  T.mid = B.alloc<int>(v6);
  T.c = B.alloc<int>(nv);
  T.off = B.alloc<int>(static_cast<size_t>(nv) + 1);
  T.sums = B.alloc<int>((static_cast<size_t>(nv) + kScanChunk - 1) / kScanChunk);
  T.ved = B.alloc<int>(v6);
  T.vtr = B.alloc<int>(v6);
  T.edv = B.alloc<int>(2 * static_cast<size_t>(ne));
  T.edsh = B.alloc<int>(2 * static_cast<size_t>(ne));
  T.trv = B.alloc<int>(3 * static_cast<size_t>(nt));
  T.tred = B.alloc<int>(3 * static_cast<size_t>(nt));
  T.counts = B.alloc<unsigned long long>(3);
  if (B.err == cudaSuccess) B.err = cudaMemset(T.counts, 0, 3 * sizeof(unsigned long long));
  if (B.err == cudaSuccess)
    B.err = cudaMemcpy(T.p, p0.data(), p0.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (B.err == cudaSuccess)
    B.err = cudaMemcpy(T.tri, t0.data(), t0.size() * sizeof(int), cudaMemcpyHostToDevice);
  auto fail = [&](cudaError_t err) {
    *why = cudaGetErrorString(err);
    return cuda_status(err);
  };
  if (B.err != cudaSuccess) return fail(B.err);
  // subdivision, level by level; every count is checked on the host before
  // the kernels that write through it run
  int n1 = 12;
  int64_t ntr = 20;
  bool ok = true;
  int total = 0;
  for (int lev = 1; lev <= level; ++lev) {
    if ((e = rings(T, n1, ntr, T.tri, &ok)) != cudaSuccess) return fail(e);
    if (!ok) return IMODEL_SWM_EINVAL;
    k_count<<<blocks(n1), kThreads>>>(n1, T.nnb, T.ring, 0, T.c);
    if ((e = scan(T, n1, &total)) != cudaSuccess) return fail(e);
    if (total != 3 * n1 - 6) return IMODEL_SWM_EINVAL;
    k_midpoints<<<blocks(n1), kThreads>>>(n1, T.nnb, T.ring, T.off, T.p, T.mid);
    k_subdivide<<<blocks(ntr), kThreads>>>(ntr, T.tri, T.nnb, T.ring, T.mid, T.tri2, T.counts);
    unsigned long long c[3];
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpy(c, T.counts, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess)
      return fail(e);
    if (c[1]) return IMODEL_SWM_EINVAL;
    std::swap(T.tri, T.tri2);
    n1 += total;
    ntr *= 4;
  }
  if (n1 != nv || ntr != nt) return IMODEL_SWM_EINVAL;
  if ((e = rings(T, nv, ntr, T.tri, &ok)) != cudaSuccess) return fail(e);
  if (!ok) return IMODEL_SWM_EINVAL;
  // meshstruct numbering (smeshpack.f90:706-862), 0-based
  k_count<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, 0, T.c);
  if ((e = scan(T, nv, &total)) != cudaSuccess) return fail(e);
  if (total != ne) return IMODEL_SWM_EINVAL;
  k_edge_numbers<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, T.off, T.ved, T.edv);
  k_edge_lookup<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, T.ved);
  k_count<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, 1, T.c);
  if ((e = scan(T, nv, &total)) != cudaSuccess) return fail(e);
  if (total != nt) return IMODEL_SWM_EINVAL;
  k_tri_numbers<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, T.off, T.vtr, T.trv);
  k_tri_lookup<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, T.vtr);
  k_tri_edges<<<blocks(nt), kThreads>>>(nt, T.nnb, T.ring, T.ved, T.trv, T.tred, T.counts);
  // an edge no node reaches keeps -1, which the range check reports
  if ((e = cudaMemset(T.edsh, 0xff, 2 * static_cast<size_t>(ne) * sizeof(int))) != cudaSuccess)
    return fail(e);
  k_edge_tris<<<blocks(nv), kThreads>>>(nv, T.nnb, T.ring, T.ved, T.vtr, T.edsh, T.counts);
  const int bv = blocks(nv), be = blocks(2 * static_cast<int64_t>(ne)),
            bt = blocks(3 * static_cast<int64_t>(nt));
  k_range_check<<<bv + be + bt, kThreads>>>(nv, ne, nt, bv, be, T.nnb, T.ring, T.ved, T.vtr,
                                             T.edv, T.edsh, T.trv, T.tred, T.counts);
  unsigned long long c[3];
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpy(c, T.counts, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return fail(e);
  if (c[0] || c[1] || c[2]) return IMODEL_SWM_EINVAL;
  // the grid's index arrays: 1-based, 0-padded, into buffers the triangle
  // and ring scratch no longer needs
  int *v_nb = T.from, *v_ed = T.to, *v_tr = T.mid;
  int *ed_v = B.alloc<int>(2 * static_cast<size_t>(ne)), *ed_sh = B.alloc<int>(2 * static_cast<size_t>(ne));
  int *tr_v = reinterpret_cast<int *>(T.tri2), *tr_ed = B.alloc<int>(3 * static_cast<size_t>(nt));
  if (B.err != cudaSuccess) return fail(B.err);
  const int b6 = blocks(static_cast<int64_t>(v6));
  k_export<<<b6 + be + bt, kThreads>>>(nv, ne, nt, b6, be, T.nnb, T.ring, T.ved, T.vtr, T.edv,
                                        T.edsh, T.trv, T.tred, v_nb, v_ed, v_tr, ed_v, ed_sh,
                                        tr_v, tr_ed);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  g.nv = nv;
  g.ne = ne;
  g.nt = nt;
  B.download(g.v_p, T.p, 3 * static_cast<size_t>(nv));
  B.download(g.nnb, T.nnb, nv);
  B.download(g.v_nb, v_nb, v6);
  B.download(g.v_ed, v_ed, v6);
  B.download(g.v_tr, v_tr, v6);
  B.download(g.ed_v, ed_v, 2 * static_cast<size_t>(ne));
  B.download(g.ed_sh, ed_sh, 2 * static_cast<size_t>(ne));
  B.download(g.tr_v, tr_v, 3 * static_cast<size_t>(nt));
  B.download(g.tr_ed, tr_ed, 3 * static_cast<size_t>(nt));
  if (B.err != cudaSuccess) return fail(B.err);
  Dev D;
  D.nv = nv;
  D.ne = ne;
  D.nt = nt;
  D.p = T.p;
  D.nnb = T.nnb;
  D.ved = T.ved;
  D.vtr = T.vtr;
  D.edv = T.edv;
  D.edsh = T.edsh;
  D.trv = T.trv;
  D.tred = T.tred;
  return geometry_dev(B, D, g, why);
}

}  // namespace mesh
}  // namespace imodel
