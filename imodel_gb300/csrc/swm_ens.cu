// Batched ensembles: several grids, each with several members, advanced by
// one persistent cooperative launch (FP32, cell-centred TRSK).
//
// Members of a grid share its geometry; their state is interleaved with the
// member index fastest (entity i, member m at i*M + m), so the threads of a
// warp that share an entity read its geometry once and the members' values
// from contiguous memory.  The kernel loops over "macro steps": the grid with
// the most steps steps every time, the others are spread evenly over the same
// macro steps.  Each RK stage is three phases (triangles, cells, edges) over
// the work of every grid that steps, separated by grid-wide barriers; each
// barrier's wait is bounded and reports a timeout through the error flag
// instead of waiting forever.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "imodel_swm.h"
#include "swm_common.cuh"
#include "swm_k32_body.cuh"
#include "swm_layout.h"

namespace imodel {
namespace {

constexpr int kMaxGrids = 8;

// Division of 0 <= n < 2^31 by an invariant d >= 1 with one multiply-high
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, fig. 4.1): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (umulhi(m, n) + n) >> l; the sum
// cannot overflow 32 bits for n < 2^31.
struct FastDiv {
  uint32_t m = 1, l = 0;
  __device__ __forceinline__ int operator()(int n) const {
    const uint32_t u = static_cast<uint32_t>(n);
    return static_cast<int>((__umulhi(m, u) + u) >> l);
  }
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  while ((1ull << f.l) < d) ++f.l;
  f.m = static_cast<uint32_t>(((1ull << 32) * ((1ull << f.l) - d)) / d + 1);
  return f;
}

struct GridDev {
  DevMesh M;
  int members;
  FastDiv per_member;  // entity index = item / members
  float h_ref;
  int nsteps;  // steps this launch
  float dt;
  float *yn_h, *yn_u, *ya_h, *ya_u, *yb_h, *yb_u, *acc_h, *acc_u;
  float *q_tr, *bern, *zflux;
};

struct EnsArgs {
  int ngrids;
  int macro_steps;
  int pv_on, mom_on;
  GridDev g[kMaxGrids];
  unsigned *bar_count;
  unsigned *bar_gen;
  int *flags;  // bit 0: PV division by ~0, bit 2: barrier timed out
  // test hook: block stall_block (-1: none) leaves before its first
  // barrier; spin_limit bounds every barrier wait (polls of ~64 ns)
  int stall_block;
  unsigned long long spin_limit;
};

// grid-wide barrier with a bounded wait (cooperative launch: all blocks are
// resident).  Returns false, with bit 2 of *flags set, if it gave up.
__device__ bool grid_barrier(const EnsArgs &A) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *gen = A.bar_gen;
    const unsigned g0 = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(A.bar_count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(A.bar_count, 0u);
      __threadfence();
      atomicAdd(A.bar_gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g0) {
        if (++spins > A.spin_limit) {  // 2^26: several seconds; a phase takes < 10 ms
          atomicOr(A.flags, 4);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool steps_now(int s, int n, int S) {
  // grid with n of S macro steps steps at s iff floor((s+1)n/S) > floor(s n/S)
  return (static_cast<long long>(s + 1) * n) / S > (static_cast<long long>(s) * n) / S;
}

// MINB = 1: registers as the compiler likes them; MINB = 2: capped at 64 per
// thread for twice the resident warps (the tuner times both)
template <int MINB>
__global__ void __launch_bounds__(512, MINB) k_ensemble(EnsArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (static_cast<int>(blockIdx.x) == A.stall_block) return;  // test hook
  for (int s = 0; s < A.macro_steps; ++s) {
    bool on[kMaxGrids];
    for (int k = 0; k < A.ngrids; ++k) on[k] = steps_now(s, A.g[k].nsteps, A.macro_steps);
    for (int st = 0; st < 4; ++st) {
      // Each phase walks the grids that step now; item r of a grid is
      // entity r / members, member r % members (all counts < 2^31).
      // phase 1: potential vorticity at triangles
      for (int k = 0; k < A.ngrids; ++k) {
        if (!on[k]) continue;
        const GridDev &G = A.g[k];
        const float *hin = st == 0 ? G.yn_h : (st == 2 ? G.yb_h : G.ya_h);
        const float *uin = st == 0 ? G.yn_u : (st == 2 ? G.yb_u : G.ya_u);
        const int n = G.M.nt * G.members;
        for (int r = tid; r < n; r += nthr) {
          const int t = G.per_member(r), m = r - t * G.members;
          tri_body<Member, LdL2>(G.M, t, Member{G.members, m}, hin, uin, G.q_tr, G.h_ref,
                                 A.pv_on, A.flags);
        }
      }
      if (!grid_barrier(A)) return;
      // phase 2: cells
      for (int k = 0; k < A.ngrids; ++k) {
        if (!on[k]) continue;
        const GridDev &G = A.g[k];
        const float *hin = st == 0 ? G.yn_h : (st == 2 ? G.yb_h : G.ya_h);
        const float *uin = st == 0 ? G.yn_u : (st == 2 ? G.yb_u : G.ya_u);
        float *hout = st == 0 ? G.ya_h : (st == 1 ? G.yb_h : (st == 2 ? G.ya_h : G.yn_h));
        const int n = G.M.nv * G.members;
        for (int r = tid; r < n; r += nthr) {
          const int i = G.per_member(r), m = r - i * G.members;
          cell_body<Member, LdL2>(G.M, i, Member{G.members, m}, hin, uin, G.q_tr, G.bern,
                                  G.zflux, G.yn_h, G.acc_h, hout, nullptr, st, G.dt,
                                  static_cast<float>(G.M.grav), G.h_ref);
        }
      }
      if (!grid_barrier(A)) return;
      // phase 3: edges
      for (int k = 0; k < A.ngrids; ++k) {
        if (!on[k]) continue;
        const GridDev &G = A.g[k];
        float *uout = st == 0 ? G.ya_u : (st == 1 ? G.yb_u : (st == 2 ? G.ya_u : G.yn_u));
        const int n = G.M.ne * G.members;
        for (int r = tid; r < n; r += nthr) {
          const int e = G.per_member(r), m = r - e * G.members;
          edge_body<Member, LdL2>(G.M, e, Member{G.members, m}, __ldg(&G.M.e_vs2[e]), G.bern,
                                  G.zflux, G.yn_u, G.acc_u, uout, nullptr, st, G.dt, A.mom_on,
                                  static_cast<float>(G.M.erad));
        }
      }
      if (!grid_barrier(A)) return;
    }
  }
}

// member m of a grid <-> reference-ordered FP64 arrays
__global__ void k_ens_gather(int n, int M, int m, const int32_t *__restrict__ n2o,
                             const double *__restrict__ src, float *__restrict__ dst, double shift) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i * M + m] = static_cast<float>(src[n2o[i]] - shift);
}
__global__ void k_ens_scatter(int n, int M, int m, const int32_t *__restrict__ n2o,
                              const float *__restrict__ src, double *__restrict__ dst,
                              double shift, int *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double v = static_cast<double>(src[i * M + m]) + shift;
    dst[n2o[i]] = v;
    if (!isfinite(v)) atomicOr(flags, 2);
  }
}

struct GridHost {
  int nv = 0, ne = 0, nt = 0, members = 0;
  bool href_fixed = false;
  double h_ref = 0.0;
  std::vector<double> areag;  // reference order
  int32_t *cell_n2o = nullptr, *edge_n2o = nullptr;
  GridDev dev{};
};

struct Ens {
  std::string err;
  int device = 0;
  int testcase = 2;
  int ngrids = 0;
  GridHost g[kMaxGrids];
  std::vector<void *> allocs;
  double *stage_h = nullptr, *stage_u = nullptr;
  unsigned *bar = nullptr;  // [0] count, [1] generation
  int *flags = nullptr;
  int *h_flags = nullptr;
  cudaStream_t stream = nullptr;
  int block = 256, blocks_per_sm = 0, variant = 0;
  bool any_state = false;
  // test hook for the next launch only (imodel_swm_ensemble_test_stall)
  int test_stall_block = -1;
  unsigned long long test_spin_limit = 0;
};

int fail(Ens *E, int code, const std::string &m) {
  E->err = m;
  return code;
}

#define EK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return imodel::fail(E, e_ == cudaErrorMemoryAllocation ? IMODEL_SWM_ENOMEM : IMODEL_SWM_ECUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

template <class V, class A>
int up(Ens *E, const std::vector<V, A> &v, const V **dst) {
  void *p = nullptr;
  EK(cudaMalloc(&p, (v.empty() ? 1 : v.size()) * sizeof(V)));
  E->allocs.push_back(p);
  if (!v.empty()) EK(cudaMemcpy(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
  *dst = static_cast<const V *>(p);
  return IMODEL_SWM_OK;
}

template <class T>
int zalloc(Ens *E, T **p, size_t n) {
  void *q = nullptr;
  EK(cudaMalloc(&q, (n ? n : 1) * sizeof(T)));
  E->allocs.push_back(q);
  EK(cudaMemset(q, 0, (n ? n : 1) * sizeof(T)));
  *p = static_cast<T *>(q);
  return IMODEL_SWM_OK;
}

int ens_create(Ens *E, const imodel_swm_mesh *meshes, int ngrids, const int32_t *members) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(E, IMODEL_SWM_ENODEV, "no CUDA device");
  if (E->device < 0 || E->device >= ndev) return fail(E, IMODEL_SWM_EINVAL, "bad device ordinal");
  EK(cudaSetDevice(E->device));
  EK(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking));
  E->ngrids = ngrids;
  size_t maxn = 0;
  int rc;
  for (int k = 0; k < ngrids; ++k) {
    if (members[k] < 1) return fail(E, IMODEL_SWM_EINVAL, "every grid needs at least one member");
    Layout L;
    std::string msg = build_layout(meshes[k], nullptr, L);
    if (!msg.empty()) return fail(E, IMODEL_SWM_EINVAL, "grid " + std::to_string(k) + ": " + msg);
    const size_t M = members[k];
    if ((static_cast<size_t>(L.ne) * M) > static_cast<size_t>(0x7FFFFFFF / 8) ||
        (static_cast<size_t>(L.nv) * 6 * M) > static_cast<size_t>(0x7FFFFFFF / 2))
      return fail(E, IMODEL_SWM_EINVAL, "grid " + std::to_string(k) + ": too many members");
    GridHost &G = E->g[k];
    G.nv = L.nv;
    G.ne = L.ne;
    G.nt = L.nt;
    G.members = members[k];
    G.areag.assign(meshes[k].hx_areag, meshes[k].hx_areag + L.nv);
    maxn = std::max(maxn, static_cast<size_t>(std::max(L.nv, L.ne)));
    DevMesh &D = G.dev.M;
    std::memset(&D, 0, sizeof(D));
    D.nv = L.nv;
    D.ne = L.ne;
    D.nt = L.nt;
    D.erad = L.erad;
    D.grav = L.grav;
    std::vector<float> bt32(L.nv, 0.0f);
    const int32_t *ra = nullptr, *rb = nullptr, *rcc = nullptr;
    if ((rc = up(E, L.t_recA, &ra)) || (rc = up(E, L.t_recB, &rb)) ||
        (rc = up(E, L.t_recC, &rcc)))
      return rc;
    D.t_recA = reinterpret_cast<const int4 *>(ra);
    D.t_recB = reinterpret_cast<const int4 *>(rb);
    D.t_recC = reinterpret_cast<const float4 *>(rcc);
    const int32_t *pk = nullptr;
    const float *kd = nullptr;
    const uint32_t *vs2 = nullptr;
    const int32_t *cn2o = nullptr, *en2o = nullptr;
    if ((rc = up(E, L.t_ed, &D.t_ed)) || (rc = up(E, L.t_v, &D.t_v)) ||
        (rc = up(E, L.t_f32, &D.t_f32)) || (rc = up(E, L.c_meta, &D.c_meta)) ||
        (rc = up(E, L.c_inva32, &D.c_inva32)) || (rc = up(E, bt32, &D.c_bt32)) ||
        (rc = up(E, L.e_grad32, &D.e_grad32)) || (rc = up(E, L.c_pk, &pk)) ||
        (rc = up(E, L.c_kd, &kd)) || (rc = up(E, L.e_vs2, &vs2)) ||
        (rc = up(E, L.cell_n2o, &cn2o)) || (rc = up(E, L.edge_n2o, &en2o)))
      return rc;
    D.c_pk = reinterpret_cast<const int4 *>(pk);
    D.c_kd = reinterpret_cast<const float2 *>(kd);
    D.e_vs2 = reinterpret_cast<const uint2 *>(vs2);
    G.cell_n2o = const_cast<int32_t *>(cn2o);
    G.edge_n2o = const_cast<int32_t *>(en2o);
    GridDev &W = G.dev;
    W.members = G.members;
    W.per_member = make_fastdiv(static_cast<uint32_t>(G.members));
    float **bv[] = {&W.yn_h, &W.ya_h, &W.yb_h, &W.acc_h, &W.bern};
    for (float **b : bv)
      if ((rc = zalloc(E, b, static_cast<size_t>(L.nv) * M))) return rc;
    float **be[] = {&W.yn_u, &W.ya_u, &W.yb_u, &W.acc_u};
    for (float **b : be)
      if ((rc = zalloc(E, b, static_cast<size_t>(L.ne) * M))) return rc;
    if ((rc = zalloc(E, &W.q_tr, static_cast<size_t>(L.nt) * M)) ||
        (rc = zalloc(E, &W.zflux, static_cast<size_t>(L.nv) * 6 * M)))
      return rc;
  }
  if ((rc = zalloc(E, &E->stage_h, maxn)) || (rc = zalloc(E, &E->stage_u, maxn)) ||
      (rc = zalloc(E, &E->bar, 2)) || (rc = zalloc(E, &E->flags, 1)))
    return rc;
  EK(cudaMallocHost(&E->h_flags, sizeof(int)));
  return IMODEL_SWM_OK;
}

int ens_flags(Ens *E) {
  EK(cudaMemcpyAsync(E->h_flags, E->flags, sizeof(int), cudaMemcpyDeviceToHost, E->stream));
  EK(cudaMemsetAsync(E->flags, 0, sizeof(int), E->stream));
  EK(cudaStreamSynchronize(E->stream));
  const int f = *E->h_flags;
  if (f & 4) return fail(E, IMODEL_SWM_ECUDA, "grid barrier timed out");
  if (f & 1) return fail(E, IMODEL_SWM_EDIVZERO, "division by zero in PV (|h_tr| < eps/1e5)");
  if (f & 2) return fail(E, IMODEL_SWM_EBLOWUP, "state holds NaN or Inf");
  return IMODEL_SWM_OK;
}

inline const void *ens_kernel(int variant) {
  return variant == 1 ? reinterpret_cast<const void *>(k_ensemble<2>)
                      : reinterpret_cast<const void *>(k_ensemble<1>);
}

int ens_launch(Ens *E, const double *dt, const int32_t *nsteps, int block, int bps,
               int variant) {
  EnsArgs A;
  std::memset(&A, 0, sizeof(A));
  A.ngrids = E->ngrids;
  A.pv_on = E->testcase >= 2 ? 1 : 0;
  A.mom_on = E->testcase > 1 ? 1 : 0;
  int S = 0;
  for (int k = 0; k < E->ngrids; ++k) {
    if (nsteps[k] < 0 || !std::isfinite(dt[k])) return fail(E, IMODEL_SWM_EINVAL, "bad dt or nsteps");
    A.g[k] = E->g[k].dev;
    A.g[k].nsteps = nsteps[k];
    A.g[k].dt = static_cast<float>(dt[k]);
    A.g[k].h_ref = static_cast<float>(E->g[k].h_ref);
    S = std::max(S, static_cast<int>(nsteps[k]));
  }
  if (S == 0) return IMODEL_SWM_OK;
  A.macro_steps = S;
  A.bar_count = E->bar;
  A.bar_gen = E->bar + 1;
  A.flags = E->flags;
  A.stall_block = E->test_stall_block;
  A.spin_limit = E->test_spin_limit ? E->test_spin_limit : (1ull << 26);
  E->test_stall_block = -1;
  E->test_spin_limit = 0;
  int dev = E->device, sms = 0, coop = 0, occ = 0;
  EK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  EK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return fail(E, IMODEL_SWM_ECUDA, "device does not support cooperative launch");
  EK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ens_kernel(variant), block, 0));
  if (occ < 1) return fail(E, IMODEL_SWM_ECUDA, "ensemble kernel does not fit an SM");
  const int per_sm = (bps > 0 && bps <= occ) ? bps : occ;
  EK(cudaMemsetAsync(E->bar, 0, 2 * sizeof(unsigned), E->stream));
  void *args[] = {&A};
  EK(cudaLaunchCooperativeKernel(ens_kernel(variant), dim3(sms * per_sm),
                                 dim3(block), args, 0, E->stream));
  return IMODEL_SWM_OK;
}

}  // namespace
}  // namespace imodel

using imodel::Ens;

extern "C" {

int imodel_swm_ensemble_create(const imodel_swm_mesh *meshes, int32_t ngrids,
                               const int32_t *members, int32_t testcase, int32_t device,
                               void **ens) {
  if (!ens) return IMODEL_SWM_EINVAL;
  *ens = nullptr;
  Ens *E = new (std::nothrow) Ens();
  if (!E) return IMODEL_SWM_ENOMEM;
  *ens = E;
  if (!meshes || !members || ngrids < 1 || ngrids > imodel::kMaxGrids)
    return imodel::fail(E, IMODEL_SWM_EINVAL, "need 1..8 grids with member counts");
  E->device = device;
  E->testcase = testcase;
  try {
    return imodel::ens_create(E, meshes, ngrids, members);
  } catch (const std::bad_alloc &) {
    return imodel::fail(E, IMODEL_SWM_ENOMEM, "host allocation failed");
  }
}

int imodel_swm_ensemble_set_state(void *ens, int32_t grid, int32_t member, const double *h,
                                  const double *u) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E || !h || !u || grid < 0 || grid >= E->ngrids) return IMODEL_SWM_EINVAL;
  imodel::GridHost &G = E->g[grid];
  if (member < 0 || member >= G.members) return imodel::fail(E, IMODEL_SWM_EINVAL, "bad member");
  if (cudaSetDevice(E->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  if (!G.href_fixed) {
    double s = 0.0, a = 0.0;
    for (int i = 0; i < G.nv; ++i) {
      a += G.areag[i];
      s += G.areag[i] * h[i];
    }
    G.h_ref = static_cast<double>(static_cast<float>(s / a));
    G.href_fixed = true;
  }
  EK(cudaMemcpyAsync(E->stage_h, h, sizeof(double) * G.nv, cudaMemcpyHostToDevice, E->stream));
  EK(cudaMemcpyAsync(E->stage_u, u, sizeof(double) * G.ne, cudaMemcpyHostToDevice, E->stream));
  imodel::k_ens_gather<<<(G.nv + 255) / 256, 256, 0, E->stream>>>(G.nv, G.members, member,
                                                                  G.cell_n2o, E->stage_h,
                                                                  G.dev.yn_h, G.h_ref);
  imodel::k_ens_gather<<<(G.ne + 255) / 256, 256, 0, E->stream>>>(G.ne, G.members, member,
                                                                  G.edge_n2o, E->stage_u,
                                                                  G.dev.yn_u, 0.0);
  EK(cudaGetLastError());
  EK(cudaStreamSynchronize(E->stream));
  E->any_state = true;
  return IMODEL_SWM_OK;
}

int imodel_swm_ensemble_get_state(void *ens, int32_t grid, int32_t member, double *h,
                                  double *u) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E || !h || !u || grid < 0 || grid >= E->ngrids) return IMODEL_SWM_EINVAL;
  imodel::GridHost &G = E->g[grid];
  if (member < 0 || member >= G.members) return imodel::fail(E, IMODEL_SWM_EINVAL, "bad member");
  if (cudaSetDevice(E->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  imodel::k_ens_scatter<<<(G.nv + 255) / 256, 256, 0, E->stream>>>(
      G.nv, G.members, member, G.cell_n2o, G.dev.yn_h, E->stage_h, G.h_ref, E->flags);
  imodel::k_ens_scatter<<<(G.ne + 255) / 256, 256, 0, E->stream>>>(
      G.ne, G.members, member, G.edge_n2o, G.dev.yn_u, E->stage_u, 0.0, E->flags);
  EK(cudaGetLastError());
  EK(cudaMemcpyAsync(h, E->stage_h, sizeof(double) * G.nv, cudaMemcpyDeviceToHost, E->stream));
  EK(cudaMemcpyAsync(u, E->stage_u, sizeof(double) * G.ne, cudaMemcpyDeviceToHost, E->stream));
  return imodel::ens_flags(E);
}

int imodel_swm_ensemble_advance(void *ens, const double *dt, const int32_t *nsteps) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E || !dt || !nsteps) return IMODEL_SWM_EINVAL;
  if (!E->any_state) return imodel::fail(E, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(E->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  int rc = imodel::ens_launch(E, dt, nsteps, E->block, E->blocks_per_sm, E->variant);
  if (rc) return rc;
  return imodel::ens_flags(E);
}

int imodel_swm_ensemble_test_stall(void *ens, int32_t block, int64_t spin_limit) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E || block < 0 || spin_limit < 1) return IMODEL_SWM_EINVAL;
  E->test_stall_block = block;
  E->test_spin_limit = static_cast<unsigned long long>(spin_limit);
  return IMODEL_SWM_OK;
}

int imodel_swm_ensemble_tune(void *ens, const double *dt, int32_t nsteps, int32_t choice[3]) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E || !dt || !choice || nsteps <= 0) return IMODEL_SWM_EINVAL;
  if (!E->any_state) return imodel::fail(E, IMODEL_SWM_ESTATE, "no state set");
  if (cudaSetDevice(E->device) != cudaSuccess) return IMODEL_SWM_ECUDA;
  // save the state of every grid, time the candidates, restore
  std::vector<void *> saved;
  std::vector<size_t> sizes;
  std::vector<float *> bufs;
  for (int k = 0; k < E->ngrids; ++k) {
    imodel::GridHost &G = E->g[k];
    bufs.push_back(G.dev.yn_h);
    sizes.push_back(sizeof(float) * G.nv * G.members);
    bufs.push_back(G.dev.yn_u);
    sizes.push_back(sizeof(float) * G.ne * G.members);
  }
  for (size_t q = 0; q < bufs.size(); ++q) {
    void *p = nullptr;
    if (cudaMalloc(&p, sizes[q]) != cudaSuccess) {
      for (void *x : saved) cudaFree(x);
      return imodel::fail(E, IMODEL_SWM_ENOMEM, "tune: no room to save the state");
    }
    saved.push_back(p);
    cudaMemcpyAsync(p, bufs[q], sizes[q], cudaMemcpyDeviceToDevice, E->stream);
  }
  std::vector<int32_t> ns(E->ngrids, nsteps);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bb = E->block, bbps = E->blocks_per_sm, bv = E->variant;
  int rc = IMODEL_SWM_OK;
  const int blocks[3] = {128, 256, 512};
  for (int v = 0; v < 2 && rc == IMODEL_SWM_OK; ++v)
    for (int b : blocks) {
      int occ = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, imodel::ens_kernel(v), b, 0);
      for (int bps = occ; bps >= 1 && rc == IMODEL_SWM_OK; bps = bps > 1 ? bps / 2 : 0) {
        cudaEventRecord(e0, E->stream);
        rc = imodel::ens_launch(E, dt, ns.data(), b, bps, v);
        cudaEventRecord(e1, E->stream);
        if (rc) break;
        rc = imodel::ens_flags(E);
        float ms = 1e30f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rc == IMODEL_SWM_OK && ms < best) {
          best = ms;
          bb = b;
          bbps = bps;
          bv = v;
        }
        if (bps == 1) break;
      }
    }
  for (size_t q = 0; q < bufs.size(); ++q)
    cudaMemcpyAsync(bufs[q], saved[q], sizes[q], cudaMemcpyDeviceToDevice, E->stream);
  cudaStreamSynchronize(E->stream);
  for (void *x : saved) cudaFree(x);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  E->block = bb;
  E->blocks_per_sm = bbps;
  E->variant = bv;
  choice[0] = bb;
  choice[1] = bbps;
  choice[2] = bv;
  return IMODEL_SWM_OK;
}

int imodel_swm_ensemble_destroy(void *ens) {
  Ens *E = static_cast<Ens *>(ens);
  if (!E) return IMODEL_SWM_OK;
  if (E->stream) cudaStreamSynchronize(E->stream);
  for (void *p : E->allocs) cudaFree(p);
  if (E->h_flags) cudaFreeHost(E->h_flags);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
  return IMODEL_SWM_OK;
}

const char *imodel_swm_ensemble_last_error(void *ens) {
  Ens *E = static_cast<Ens *>(ens);
  return E ? E->err.c_str() : "NULL handle";
}

void *imodel_swm_ensemble_stream(void *ens) {
  Ens *E = static_cast<Ens *>(ens);
  return E ? static_cast<void *>(E->stream) : nullptr;
}

}  // extern "C"
