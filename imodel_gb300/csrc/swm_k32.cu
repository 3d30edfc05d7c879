// FP32 kernels of the TRSK shallow-water step.
//
// Same data flow as the FP64 kernels (triangle -> edge -> cell -> edge per
// RK stage), with every constant factor of a term folded into one
// coefficient computed in FP64 and rounded once, and the thickness stored as
// a deviation from a constant reference depth h_ref so that the FP32 state
// keeps ~1e-5 m resolution on ~3 km deep layers.
#include "swm_common.cuh"

namespace imodel {
namespace {

__device__ __forceinline__ float rk_stage32(int stage, float k, float yn, float *acc, float dt) {
  // ode_rk4, swm.f90:2647-2678
  if (stage == 0) {
    *acc = k;
    return yn + 0.5f * dt * k;
  } else if (stage == 1) {
    *acc = *acc + 2.0f * k;
    return yn + 0.5f * dt * k;
  } else if (stage == 2) {
    *acc = *acc + 2.0f * k;
    return yn + dt * k;
  }
  return yn + dt * (*acc + k) * (1.0f / 6.0f);
}

// q_t = (curl u / A + f) / h_t  (vort_tr + scalar_hx2tr + scalar_elem_divide)
__global__ void __launch_bounds__(512) k_tri32(DevMesh M, const float *__restrict__ hd,
                                               const float *__restrict__ u,
                                               float *__restrict__ q_tr, float h_ref,
                                               int pv_on, int *flags) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.nt;
  if (t >= nt) return;
  float eta = M.t_f32[t];
  float ht = 0.0f;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    eta += __ldg(&M.t_circ32[s * nt + t]) * u[__ldg(&M.t_ed[s * nt + t])];
    ht += __ldg(&M.t_kite32[s * nt + t]) * hd[__ldg(&M.t_v[s * nt + t])];
  }
  ht += h_ref;
  float q = 0.0f;
  if (pv_on) {
    // scalar_elem_divide guard, swm_operators.f90:1604-1606
    if (fabsf(ht) < 1.1920928955078125e-12f)
      atomicOr(flags, 1);
    else
      q = eta / ht;
  }
  q_tr[t] = q;
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

// ---- cell-centred TRSK (variant 1) ------------------------------------------
//
// coriolis_ed (swm_operators.f90:1283-1308) sums, for edge e and each of its
// two cells c, over the other edges k_j of c:
//     F_k * (q_e + q_k)/2 * d_k * w_c(i_e, j) * ttgout_c(j) * tnrccw_c(i_e)
// with w_c(i, j) = sum_{k=i}^{j-1} R_c(k) - 1/2 (calc_trisk_weights,
// interpack.f90:4046-4095).  Every factor but q_e lives on cell c, so each
// cell computes the contribution Z_c(i) of all its n edges at once from its n
// kite fractions R_c; the edge kernel adds the two cells' Z and divides by
// l_e.  The 10-entry stencil (40 B of indices and 40 B of weights per edge)
// becomes n fractions per cell.
template <int N>
__device__ __forceinline__ void trsk_cell(const float (&G)[6], const float (&qs)[6],
                                          const float (&R)[6], unsigned tneg, float (&Z)[6]) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float c = 0.0f, acc = 0.0f;
#pragma unroll
    for (int s = 1; s < N; ++s) {
      const int j = (i + s) % N;
      c += R[(i + s - 1) % N];
      acc += (c - 0.5f) * G[j] * (qs[i] + qs[j]);
    }
    const float z = 0.5f * acc;
    Z[i] = ((tneg >> i) & 1u) ? -z : z;
  }
}

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
  const int nv = M.nv;
  if (i >= nv) return;
  const uint32_t meta = __ldg(&M.c_meta[i]);
  const int n = static_cast<int>(meta & 7u);
  const unsigned tneg = meta >> 8;
  const float hi = hd[i];
  float G[6], qs[6], R[6];
  float div = 0.0f, ke = 0.0f;
  float qprev = q_tr[__ldg(&M.c_tr[(n - 1) * nv + i])];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    G[j] = 0.0f;
    qs[j] = 0.0f;
    R[j] = 0.0f;
    if (j < n) {
      const int e = __ldg(&M.c_ed[j * nv + i]);
      const int nb = __ldg(&M.c_nb[j * nv + i]);
      const int t = __ldg(&M.c_tr[j * nv + i]);
      const float ue = u[e];
      // F_e = u_e h_e with h_e the two-cell average (scalar_hx2ed)
      const float F = ue * (h_ref + 0.5f * (hi + hd[nb]));
      G[j] = F * __ldg(&M.c_dg32[j * nv + i]);
      // q_e: edge j lies between triangles j-1 and j (scalar_tr2ed)
      const float qt = q_tr[t];
      qs[j] = 0.5f * (qprev + qt);
      qprev = qt;
      R[j] = __ldg(&M.c_R32[j * nv + i]);
      div += G[j];
      ke += __ldg(&M.c_kew32[j * nv + i]) * (ue * ue);
    }
  }
  bern[i] = grav * (hi + __ldg(&M.c_bt32[i])) + ke;
  float Z[6];
  if (n == 6)
    trsk_cell<6>(G, qs, R, tneg, Z);
  else if (n == 5)
    trsk_cell<5>(G, qs, R, tneg, Z);
  else if (n == 4)
    trsk_cell<4>(G, qs, R, tneg, Z);
  else
    trsk_cell<3>(G, qs, R, tneg, Z);
#pragma unroll
  for (int j = 0; j < 6; ++j)
    if (j < n) zflux[j * nv + i] = Z[j];
  const float masseq = -div * __ldg(&M.c_inva32[i]);
  if (stage < 0)
    tend[i] = masseq;
  else
    yout[i] = rk_stage32(stage, masseq, yn[i], acc + i, dt);
}

// -grad B - (Z_c1 + Z_c2) / l_e and the momentum RK stage
__global__ void __launch_bounds__(512) k_edge32v2(DevMesh M, const float *__restrict__ bern,
                                                  const float *__restrict__ zflux,
                                                  const float *__restrict__ yn,
                                                  float *__restrict__ acc,
                                                  float *__restrict__ yout,
                                                  float *__restrict__ tend, int stage, float dt,
                                                  int mom_on, float erad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne, nv = M.nv;
  if (e >= ne) return;
  const uint32_t w1 = __ldg(&M.e_vs[e]), w2 = __ldg(&M.e_vs[ne + e]);
  const int c1 = static_cast<int>(w1 & 0x0FFFFFFFu), c2 = static_cast<int>(w2 & 0x0FFFFFFFu);
  const int s1 = static_cast<int>(w1 >> 28), s2 = static_cast<int>(w2 >> 28);
  const float g = __ldg(&M.e_grad32[e]);  // 1 / (l_e a)
  const float grad = (bern[c2] - bern[c1]) * g;
  const float q = (zflux[s1 * nv + c1] + zflux[s2 * nv + c2]) * (g * erad);
  float momeq = -grad - q;
  if (!mom_on) momeq = 0.0f;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage32(stage, momeq, yn[e], acc + e, dt);
}

inline int nblocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void launch_stage32(const DevMesh &M, const Work<float> &W, const float *h_in,
                    const float *u_in, float *h_out, float *u_out, int stage, float dt,
                    cudaStream_t s, cudaEvent_t *ev) {
  const Tune &T = W.tune;
  const float grav = static_cast<float>(M.grav);
  if (ev) cudaEventRecord(ev[0], s);
  k_tri32<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ref, W.pv_on,
                                                        W.flags);
  if (T.variant == 1) {
    if (ev) cudaEventRecord(ev[1], s);
    if (ev) cudaEventRecord(ev[2], s);
    k_cell32v2<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
        M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
        grav, W.h_ref);
    if (ev) cudaEventRecord(ev[3], s);
    k_edge32v2<<<nblocks(M.ne, T.bs_edge), T.bs_edge, 0, s>>>(
        M, W.bern, W.zflux, W.yn_u, W.acc_u, u_out, W.tend_u, stage, dt, W.mom_on,
        static_cast<float>(M.erad));
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
