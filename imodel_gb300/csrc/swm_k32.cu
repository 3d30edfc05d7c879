// FP32 kernels of the TRSK shallow-water step.
//
// Same data flow as the FP64 kernels (triangle -> edge -> cell -> edge per
// RK stage), with every constant factor of a term folded into one
// coefficient computed in FP64 and rounded once, and the thickness stored as
// a deviation from a constant reference depth h_ref so that the FP32 state
// keeps ~1e-5 m resolution on ~3 km deep layers.
#include "swm_k32_body.cuh"

namespace imodel {
namespace {

// q_t = (curl u / A + f) / h_t  (vort_tr + scalar_hx2tr + scalar_elem_divide)
__global__ void __launch_bounds__(512) k_tri32(DevMesh M, const float *__restrict__ hd,
                                               const float *__restrict__ u,
                                               float *__restrict__ q_tr, float h_ref,
                                               int pv_on, int *flags) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.nt) return;
  tri_body(M, t, OneRun{}, hd, u, q_tr, h_ref, pv_on, flags);
}

// h_e (deviation), flux F_e = u_e (h_ref + h_e), q_e
__global__ void __launch_bounds__(512) k_edge_pre32(DevMesh M, const float *__restrict__ hd,
                                                    const float *__restrict__ u,
                                                    const float *__restrict__ q_tr,
                                                    float *__restrict__ h_ed,
                                                    float *__restrict__ uh,
                                                    float *__restrict__ q_ed, float h_ref) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const float he = 0.5f * (hd[__ldg(&M.e_v[e])] + hd[__ldg(&M.e_v[ne + e])]);
  h_ed[e] = he;
  uh[e] = u[e] * (h_ref + he);
  q_ed[e] = 0.5f * (q_tr[__ldg(&M.e_sh[e])] + q_tr[__ldg(&M.e_sh[ne + e])]);
}

// -div F, K, Bernoulli potential g (h - h_ref + b) + K, mass RK stage
__global__ void __launch_bounds__(512) k_cell32(DevMesh M, const float *__restrict__ hd,
                                                const float *__restrict__ u,
                                                const float *__restrict__ uh,
                                                float *__restrict__ bern,
                                                const float *__restrict__ yn,
                                                float *__restrict__ acc,
                                                float *__restrict__ yout,
                                                float *__restrict__ tend, int stage, float dt,
                                                float grav) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  const int n = M.c_nnb[i];
  float d = 0.0f, k = 0.0f;
  for (int j = 0; j < n; ++j) {
    const int e = __ldg(&M.c_ed[j * nv + i]);
    const float ue = u[e];
    d += __ldg(&M.c_div32[j * nv + i]) * uh[e];
    k += __ldg(&M.c_kew32[j * nv + i]) * (ue * ue);
  }
  bern[i] = grav * (hd[i] + __ldg(&M.c_bt32[i])) + k;
  const float masseq = -d;
  if (stage < 0)
    tend[i] = masseq;
  else
    yout[i] = rk_stage32(stage, masseq, yn[i], acc + i, dt);
}

// -grad B - TRSK PV flux, momentum RK stage
__global__ void __launch_bounds__(512) k_edge32(DevMesh M, const float *__restrict__ bern,
                                                const float *__restrict__ uh,
                                                const float *__restrict__ q_ed,
                                                const float *__restrict__ yn,
                                                float *__restrict__ acc,
                                                float *__restrict__ yout,
                                                float *__restrict__ tend, int stage, float dt,
                                                int mom_on) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const float g = (bern[__ldg(&M.e_v[ne + e])] - bern[__ldg(&M.e_v[e])]) * __ldg(&M.e_grad32[e]);
  const float qe = q_ed[e];
  const int ns = M.e_nst[e];
  float q = 0.0f;
  for (int s = 0; s < ns; ++s) {
    const int k = __ldg(&M.e_stk[s * ne + e]);
    q += __ldg(&M.e_stc32[s * ne + e]) * uh[k] * (qe + q_ed[k]);
  }
  float momeq = -g - q;
  if (!mom_on) momeq = 0.0f;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage32(stage, momeq, yn[e], acc + e, dt);
}

// ---- cell-centred TRSK (variant 1), bodies in swm_k32_body.cuh ------------
__global__ void __launch_bounds__(512) k_cell32v2(DevMesh M, const float *__restrict__ hd,
                                                  const float *__restrict__ u,
                                                  const float *__restrict__ q_tr,
                                                  float *__restrict__ bern,
                                                  float *__restrict__ zflux,
                                                  const float *__restrict__ yn,
                                                  float *__restrict__ acc,
                                                  float *__restrict__ yout,
                                                  float *__restrict__ tend, int stage, float dt,
                                                  float grav, float h_ref) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.nv) return;
  cell_body(M, i, OneRun{}, hd, u, q_tr, bern, zflux, yn, acc, yout, tend, stage, dt, grav, h_ref);
}

// the momentum tendency of edge e (edge_body's arithmetic): -grad B -
// (Z_c1 + Z_c2) / l_e, plus the learned correction term
__device__ __forceinline__ float edge_momeq(uint32_t wa, uint32_t wb, float g,
                                           const float *__restrict__ bern,
                                           const float *__restrict__ zflux, float erad) {
  const int c1 = static_cast<int>(wa & 0x0FFFFFFFu), c2 = static_cast<int>(wb & 0x0FFFFFFFu);
  const int s1 = static_cast<int>(wa >> 28), s2 = static_cast<int>(wb >> 28);
  const float grad = (bern[c2] - bern[c1]) * g;
  const float q = (zflux[6 * c1 + s1] + zflux[6 * c2 + s2]) * (g * erad);
  return -grad - q;
}

// ---- variant 2: the same kernels on records with 16-bit indices ---------
__global__ void __launch_bounds__(512) k_tri32c(DevMesh M, const float *__restrict__ hd,
                                                const float *__restrict__ u,
                                                float *__restrict__ q_tr, float h_ref,
                                                int pv_on, int *flags) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.nt) return;
  tri_body16(M, t, hd, u, q_tr, h_ref, pv_on, flags);
}

__global__ void __launch_bounds__(512) k_cell32c(DevMesh M, const float *__restrict__ hd,
                                                 const float *__restrict__ u,
                                                 const float *__restrict__ q_tr,
                                                 float *__restrict__ bern,
                                                 float *__restrict__ zflux,
                                                 const float *__restrict__ yn,
                                                 float *__restrict__ acc,
                                                 float *__restrict__ yout,
                                                 float *__restrict__ tend, int stage, float dt,
                                                 float grav, float h_ref) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.nv) return;
  cell_body16(M, i, hd, u, q_tr, bern, zflux, yn, acc, yout, tend, stage, dt, grav, h_ref);
}

// ---- variant 3: persistent cell kernel, software-pipelined -------------
// Each thread walks its cells with a grid stride in a three-stage pipeline
// through shared memory: while it computes cell k, the records of cell k+2
// (16-bit slot records, meta, own values, warp bases) and the 18 gathered
// values of cell k+1 (u, neighbour h, q at the triangles) are in flight as
// cp.async copies.  A thread reads back only what it copied itself, except
// the warp's index bases, which lane 0 copies.
constexpr int kPB = 128;  // threads per block
struct CellRec {
  float4 rec[6][kPB];   // 16-bit slot records
  uint32_t toff[3][kPB];
  uint32_t meta[kPB];
  float own[5][kPB];    // h deviation, b, 1/(A a), y_n, RK accumulator
  int4 wb[kPB / 32];    // warp bases
};
struct CellGather {
  float ue[6][kPB], hn[6][kPB], qt[6][kPB];
};
struct CellPipe {
  CellRec r[2];
  CellGather g[2];
};
constexpr size_t kCellPipeBytes = sizeof(CellPipe);

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(kPB) k_cell32p(DevMesh M, const float *__restrict__ hd,
                                                 const float *__restrict__ u,
                                                 const float *__restrict__ q_tr,
                                                 float *__restrict__ bern,
                                                 float *__restrict__ zflux,
                                                 const float *__restrict__ yn,
                                                 float *__restrict__ acc,
                                                 float *__restrict__ yout,
                                                 float *__restrict__ tend, int stage, float dt,
                                                 float grav, float h_ref) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CellPipe &P = *reinterpret_cast<CellPipe *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nv = M.nv;
  const int stride = gridDim.x * kPB;
  // stage 1: the records of cell c (every address checked against nv)
  auto issue_rec = [&](CellRec &B, int c) {
    if (c < nv) {
#pragma unroll
      for (int j = 0; j < 6; ++j) cp_async16(&B.rec[j][tid], &M.c_rec[j * nv + c]);
#pragma unroll
      for (int k = 0; k < 3; ++k) cp_async4(&B.toff[k][tid], &M.c_toff[k * nv + c]);
      cp_async4(&B.meta[tid], &M.c_meta[c]);
      cp_async4(&B.own[0][tid], hd + c);
      cp_async4(&B.own[1][tid], &M.c_bt32[c]);
      cp_async4(&B.own[2][tid], &M.c_inva32[c]);
      if (stage >= 0) cp_async4(&B.own[3][tid], yn + c);
      if (stage >= 1) cp_async4(&B.own[4][tid], acc + c);
      if (lane == 0) cp_async16(&B.wb[warp], &M.c_wb[c >> 5]);
    }
    cp_async_commit();
  };
  // stage 2: decode cell c's indices from its records, copy its gathers
  auto issue_gather = [&](const CellRec &B, CellGather &G, int c) {
    if (c < nv) {
      const int4 wb = B.wb[warp];
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        int e, n, t;
        if (wb.w) {
          const uint32_t w = __float_as_uint(B.rec[j][tid].w);
          const uint32_t tp = B.toff[j >> 1][tid];
          e = wb.x + static_cast<int>(w & 0xFFFFu);
          n = wb.y + static_cast<int>(w >> 16);
          t = wb.z + static_cast<int>((tp >> (16 * (j & 1))) & 0xFFFFu);
        } else {
          const int4 pk = __ldg(&M.c_pk[j * nv + c]);
          e = pk.x;
          n = pk.y;
          t = pk.z;
        }
        cp_async4(&G.ue[j][tid], u + e);
        cp_async4(&G.hn[j][tid], hd + n);
        cp_async4(&G.qt[j][tid], q_tr + t);
      }
    }
    cp_async_commit();
  };
  int base = blockIdx.x * kPB;
  // prologue: records of cells 0 and 1 in flight, gathers of cell 0
  issue_rec(P.r[0], base + tid);
  issue_rec(P.r[1], base + stride + tid);
  cp_async_wait<1>();
  __syncwarp();
  issue_gather(P.r[0], P.g[0], base + tid);
  // the trip count is uniform over a warp (its first cell decides); at the
  // top of iteration k the copies of records k+1 and gathers k are pending
  for (int k = 0; base + 32 * warp < nv; ++k, base += stride) {
    const int i = base + tid;
    CellRec &rk = P.r[k & 1];
    // cell k's record values into registers: its buffer takes cell k+2
    const uint32_t meta = rk.meta[tid];
    float R[6];
    float2 kd[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const float4 r = rk.rec[j][tid];
      R[j] = r.z;
      kd[j] = make_float2(r.x, r.y);
    }
    const float hi = rk.own[0][tid], bt = rk.own[1][tid], inva = rk.own[2][tid];
    const float ynv = stage >= 0 ? rk.own[3][tid] : 0.0f;
    const float accv = stage >= 1 ? rk.own[4][tid] : 0.0f;
    __syncwarp();  // every lane is done with the warp bases of this buffer
    issue_rec(rk, i + 2 * stride);
    cp_async_wait<1>();  // records k+1 and gathers k are in
    __syncwarp();        // lane 0's copy of the warp bases of k+1
    issue_gather(P.r[(k + 1) & 1], P.g[(k + 1) & 1], i + stride);
    if (i < nv) {
      const CellGather &gk = P.g[k & 1];
      float ue[6], hn[6], qt[6];
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        ue[j] = gk.ue[j][tid];
        hn[j] = gk.hn[j][tid];
        qt[j] = gk.qt[j][tid];
      }
      cell_math(i, meta, R, kd, ue, hn, qt, hi, bt, inva, ynv, accv, bern, zflux, acc, yout,
                tend, stage, dt, grav, h_ref);
    }
  }
  // no copy may still be writing this block's shared memory when it exits
  cp_async_wait<0>();
}

// two consecutive edges per thread: one 16-byte load of their cell words,
// 8-byte loads and stores of their per-edge values, and twice the
// independent gathers in flight
__global__ void __launch_bounds__(512) k_edge32v2(DevMesh M, const float *__restrict__ bern,
                                                  const float *__restrict__ zflux,
                                                  const float *__restrict__ yn,
                                                  float *__restrict__ acc,
                                                  float *__restrict__ yout,
                                                  float *__restrict__ tend, int stage, float dt,
                                                  int mom_on, float erad,
                                                  const float *__restrict__ corr) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int e0 = 2 * p;
  if (e0 >= M.ne) return;
  if (e0 + 1 < M.ne) {
    const uint4 w = __ldg(reinterpret_cast<const uint4 *>(M.e_vs2) + p);
    const float2 g = __ldg(reinterpret_cast<const float2 *>(M.e_grad32) + p);
    float m0 = edge_momeq(w.x, w.y, g.x, bern, zflux, erad);
    float m1 = edge_momeq(w.z, w.w, g.y, bern, zflux, erad);
    // learned correction of the PV flux (frozen over the RK step)
    if (corr) {
      const float2 c = reinterpret_cast<const float2 *>(corr)[p];
      m0 += c.x;
      m1 += c.y;
    }
    if (!mom_on) m0 = m1 = 0.0f;
    if (stage < 0) {
      reinterpret_cast<float2 *>(tend)[p] = make_float2(m0, m1);
    } else {
      const float2 y = reinterpret_cast<const float2 *>(yn)[p];
      // stage 0 only writes the accumulator
      float2 a = stage == 0 ? make_float2(0.0f, 0.0f) : reinterpret_cast<float2 *>(acc)[p];
      const float o0 = rk_stage32(stage, m0, y.x, &a.x, dt);
      const float o1 = rk_stage32(stage, m1, y.y, &a.y, dt);
      if (stage < 3) reinterpret_cast<float2 *>(acc)[p] = a;
      reinterpret_cast<float2 *>(yout)[p] = make_float2(o0, o1);
    }
  } else {
    edge_body(M, e0, OneRun{}, __ldg(&M.e_vs2[e0]), bern, zflux, yn, acc, yout, tend, stage, dt,
              mom_on, erad, corr);
  }
}

inline int nblocks(int n, int t) { return (n + t - 1) / t; }

// persistent grid of the prefetching cell kernel: the resident blocks of
// every SM (measured once), at most one block per 128 cells
int cell32p_grid(int nv) {
  static int per_sm = 0, sms = 0;
  if (per_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_cell32p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kCellPipeBytes));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cell32p, kPB, kCellPipeBytes);
    if (per_sm < 1) per_sm = 1;
    if (sms < 1) sms = 1;
  }
  const int g = per_sm * sms, need = nblocks(nv, kPB);
  return g < need ? g : need;
}

}  // namespace

void launch_stage32(const DevMesh &M, const Work<float> &W, const float *h_in,
                    const float *u_in, float *h_out, float *u_out, int stage, float dt,
                    cudaStream_t s, cudaEvent_t *ev) {
  const Tune &T = W.tune;
  const float grav = static_cast<float>(M.grav);
  if (ev) cudaEventRecord(ev[0], s);
  if (T.variant >= 2)
    k_tri32c<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ref,
                                                           W.pv_on, W.flags);
  else
    k_tri32<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ref,
                                                          W.pv_on, W.flags);
  if (T.variant >= 1) {
    if (ev) cudaEventRecord(ev[1], s);
    // learned correction: formed once per step from the first stage's state
    if (W.learned && stage <= 0)
      learned_launch(M, *W.learned, h_in, u_in, W.q_tr, W.h_ref, T.mlp_gather, W.flags, s);
    if (ev) cudaEventRecord(ev[2], s);
    if (T.variant == 3)
      k_cell32p<<<cell32p_grid(M.nv), kPB, kCellPipeBytes, s>>>(M, h_in, u_in, W.q_tr, W.bern, W.zflux,
                                                  W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
                                                  grav, W.h_ref);
    else if (T.variant == 2)
      k_cell32c<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref);
    else
      k_cell32v2<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref);
    if (ev) cudaEventRecord(ev[3], s);
    k_edge32v2<<<nblocks((M.ne + 1) / 2, T.bs_edge), T.bs_edge, 0, s>>>(
        M, W.bern, W.zflux, W.yn_u, W.acc_u, u_out, W.tend_u, stage, dt, W.mom_on,
        static_cast<float>(M.erad), W.learned ? W.learned->corr : nullptr);
    if (ev) cudaEventRecord(ev[4], s);
    return;
  }
  if (ev) cudaEventRecord(ev[1], s);
  k_edge_pre32<<<nblocks(M.ne, T.bs_pre), T.bs_pre, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ed, W.uh,
                                                             W.q_ed, W.h_ref);
  if (ev) cudaEventRecord(ev[2], s);
  k_cell32<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(M, h_in, u_in, W.uh, W.bern, W.yn_h,
                                                           W.acc_h, h_out, W.tend_h, stage, dt,
                                                           grav);
  if (ev) cudaEventRecord(ev[3], s);
  k_edge32<<<nblocks(M.ne, T.bs_edge), T.bs_edge, 0, s>>>(M, W.bern, W.uh, W.q_ed, W.yn_u,
                                                           W.acc_u, u_out, W.tend_u, stage, dt,
                                                           W.mom_on);
  if (ev) cudaEventRecord(ev[4], s);
}

}  // namespace imodel
