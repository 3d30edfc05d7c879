// GPU back end of the grid builder's geometry: meshstruct's per-entity
// geometry (smeshpack.f90:706-1151), the kite areas (trhx_intersec_areas
// :5080-5154, hxtr_intersec_areas :4991-5078), calc_trisk_weights
// (interpack.f90:3978-4098) and the Delaunay check, one thread per node,
// edge, triangle or cell, from the topology mesh.cpp builds on the host.
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

}  // namespace

int geometry_gpu(const Topo &T, Grid &g, int device, const char **why) {
  *why = "";
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return IMODEL_SWM_ECUDA;
  }
  const int nv = T.nv, ne = T.ne, nt = T.nt;
  const size_t v6 = 6 * static_cast<size_t>(nv), e3 = 3 * static_cast<size_t>(ne),
               t3 = 3 * static_cast<size_t>(nt);
  Buffers B;
  Dev D;
  D.nv = nv;
  D.ne = ne;
  D.nt = nt;
  D.p = B.upload(T.p);
  D.nnb = B.upload(T.nnb);
  D.ved = B.upload(T.ved);
  D.vtr = B.upload(T.vtr);
  D.edv = B.upload(T.edv);
  D.edsh = B.upload(T.edsh);
  D.trv = B.upload(T.trv);
  D.tred = B.upload(T.tred);
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

}  // namespace mesh
}  // namespace imodel
