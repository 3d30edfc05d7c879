// FP32 kernels of the TRSK shallow-water step.
//
// Same data flow as the FP64 kernels (triangle -> edge -> cell -> edge per
// RK stage), with every constant factor of a term folded into one
// coefficient computed in FP64 and rounded once, and the thickness stored as
// a deviation from a constant reference depth h_ref so that the FP32 state
// keeps ~1e-5 m resolution on ~3 km deep layers.
#include "imodel_swm.h"
#include "swm_k32_body.cuh"

namespace imodel {
namespace {

// q_t = (curl u / A + f) / h_t  (vort_tr + scalar_hx2tr + scalar_elem_divide)
__global__ void __launch_bounds__(512) k_tri32(DevMesh M, const float *__restrict__ hd,
                                               const float *__restrict__ u,
                                               float *__restrict__ q_tr, float h_ref,
                                               int pv_on, int *flags,
                                               const float *__restrict__ kt,
                                               float *__restrict__ coefvort,
                                               float *__restrict__ ht_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.nt) return;
  tri_body(M, t, OneRun{}, hd, u, q_tr, h_ref, pv_on, flags, kt, coefvort, ht_out);
}

// h_e (deviation), flux F_e = u_e (h_ref + h_e), q_e: the TRSK average
// (scalar_tr2ed), the circumcentre-distance weights of pxt16 (qw) or
// gass18's rhombus PV (qw and the triangle depths ht: (w1 eta1 + w2 eta2) /
// (w1 h1 + w2 h2), eta = q h, with scalar_elem_divide's guard)
__global__ void __launch_bounds__(512) k_edge_pre32(DevMesh M, const float *__restrict__ hd,
                                                    const float *__restrict__ u,
                                                    const float *__restrict__ q_tr,
                                                    float *__restrict__ h_ed,
                                                    float *__restrict__ uh,
                                                    float *__restrict__ q_ed, float h_ref,
                                                    const float *__restrict__ qg,
                                                    const float *__restrict__ vhx,
                                                    float coef,
                                                    const float *__restrict__ qw,
                                                    const float *__restrict__ ht, int pv_on,
                                                    int *flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const int c1 = __ldg(&M.e_v[e]), c2 = __ldg(&M.e_v[ne + e]);
  const float he = 0.5f * (hd[c1] + hd[c2]);
  h_ed[e] = he;
  uh[e] = u[e] * (h_ref + he);
  const int t1 = __ldg(&M.e_sh[e]), t2 = __ldg(&M.e_sh[ne + e]);
  float q;
  if (!qw) {
    q = 0.5f * (q_tr[t1] + q_tr[t2]);
  } else if (!ht) {
    q = __ldg(&qw[e]) * q_tr[t1] + __ldg(&qw[ne + e]) * q_tr[t2];
  } else {
    const float w1 = __ldg(&qw[e]), w2 = __ldg(&qw[ne + e]);
    const float h1 = ht[t1], h2 = ht[t2];
    const float hr = w1 * h1 + w2 * h2;
    q = 0.0f;
    if (pv_on) {
      if (fabsf(hr) < 1.1920928955078125e-12f)
        atomicOr(flags, 1);
      else
        q = (w1 * q_tr[t1] * h1 + w2 * q_tr[t2] * h2) / hr;
    }
  }
  if (qg) {
    // apvm (swm_operators.f90:1495-1502), coef = pvspar dt
    const int nt = M.nt, nv = M.nv;
    float d = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      d += (qg[k * nt + t1] + qg[k * nt + t2]) * (vhx[k * nv + c1] + vhx[k * nv + c2]);
    q -= coef * d;
  }
  q_ed[e] = q;
}

// The two reconstructions apvm reads, in FP32 with the layout's weights
// (swm_layout.h): blocks [0, nbt) the PV gradient at the triangles,
// vector_edtr2tr_perot (:408-452) of grad_tr2ed(q_tr) (:1427-1463); the
// blocks after the velocity at the cells, vector_edhx2hx_perot (:454-509);
// each then projected on the tangent plane of its unit point.
__global__ void __launch_bounds__(256) k_apvm32(DevMesh M, const float *__restrict__ q_tr,
                                                const float *__restrict__ u,
                                                float *__restrict__ qg,
                                                float *__restrict__ vhx, int nbt) {
  const int ne = M.ne;
  float v[3] = {0.0f, 0.0f, 0.0f}, p[3];
  int n, i, stride;
  float *out;
  if (static_cast<int>(blockIdx.x) < nbt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = M.nt;
    if (t >= nt) return;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int ed = __ldg(&M.t_ed[s * nt + t]);
      const float g = __ldg(&M.e_gtg32[ed]) *
                      (q_tr[__ldg(&M.e_sh[ne + ed])] - q_tr[__ldg(&M.e_sh[ed])]);
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = fmaf(g, __ldg(&M.t_apw32[(3 * s + k) * nt + t]), v[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = __ldg(&M.t_cc32[k * nt + t]);
    i = t;
    stride = nt;
    out = qg;
  } else {
    const int c = (blockIdx.x - nbt) * blockDim.x + threadIdx.x;
    const int nv = M.nv;
    if (c >= nv) return;
    n = M.c_nnb[c];
    for (int j = 0; j < n; ++j) {
      const float ue = u[__ldg(&M.c_ed[j * nv + c])];
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = fmaf(ue, __ldg(&M.c_apw32[(3 * j + k) * nv + c]), v[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = __ldg(&M.c_p32[k * nv + c]);
    i = c;
    stride = nv;
    out = vhx;
  }
  // proj_vec_sphere (smeshpack.f90:4419-4433) with |p| = 1
  const float vp = v[0] * p[0] + v[1] * p[1] + v[2] * p[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k * stride + i] = v[k] - vp * p[k];
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
                                                float grav, int perot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  const int n = M.c_nnb[i];
  float d = 0.0f, k = 0.0f;
  float v[3] = {0.0f, 0.0f, 0.0f};
  for (int j = 0; j < n; ++j) {
    const int e = __ldg(&M.c_ed[j * nv + i]);
    const float ue = u[e];
    d += __ldg(&M.c_div32[j * nv + i]) * uh[e];
    if (perot) {
#pragma unroll
      for (int c = 0; c < 3; ++c) v[c] = fmaf(ue, __ldg(&M.c_apw32[(3 * j + c) * nv + i]), v[c]);
    } else {
      k += __ldg(&M.c_kew32[j * nv + i]) * (ue * ue);
    }
  }
  if (perot) {
    // kinetic_energy_hx, perhx branch (pxt16): half the squared Perot
    // velocity of the cell (vector_edhx2hx_perot), on the tangent plane
    const float p0 = __ldg(&M.c_p32[i]), p1 = __ldg(&M.c_p32[nv + i]), p2 = __ldg(&M.c_p32[2 * nv + i]);
    const float vp = v[0] * p0 + v[1] * p1 + v[2] * p2;
    const float a0 = v[0] - vp * p0, a1 = v[1] - vp * p1, a2 = v[2] - vp * p2;
    k = 0.5f * (a0 * a0 + a1 * a1 + a2 * a2);
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
                                                int mom_on, const float *__restrict__ dif1,
                                                const float *__restrict__ dif2,
                                                const int32_t *__restrict__ stq,
                                                const float *__restrict__ q_tr, int dtred) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const float g = (bern[__ldg(&M.e_v[ne + e])] - bern[__ldg(&M.e_v[e])]) * __ldg(&M.e_grad32[e]);
  float q = 0.0f;
  if (dtred) {
    // coriolis_ed's dtred branch: the Perot reconstructions of F q at the
    // edge's two triangles, as six coefficients on their edges' fluxes
    const int nt = M.nt;
#pragma unroll
    for (int si = 0; si < 2; ++si) {
      const int t = __ldg(&M.e_sh[si * ne + e]);
      float a = 0.0f;
#pragma unroll
      for (int s = 0; s < 3; ++s)
        a += __ldg(&M.e_dtc32[(3 * si + s) * ne + e]) * uh[__ldg(&M.t_ed[s * nt + t])];
      q += q_tr[t] * a;
    }
  } else {
    // TRSK (trsk10, dtred's q_e aside), pered as coefficients on the same
    // stencil (pxt16), or with gass18's connecting-edge PV (stq)
    const float qe = q_ed[e];
    const int ns = M.e_nst[e];
    for (int s = 0; s < ns; ++s) {
      const int k = __ldg(&M.e_stk[s * ne + e]);
      const int c3 = stq ? __ldg(&stq[s * ne + e]) : -1;
      const float qs = c3 >= 0 ? q_ed[c3] + q_ed[c3] : qe + q_ed[k];
      q += __ldg(&M.e_stc32[s * ne + e]) * uh[k] * qs;
    }
  }
  float momeq = -g - q;
  if (dif1) momeq += dif1[e];
  if (dif2) momeq -= dif2[e];
  if (!mom_on) momeq = 0.0f;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage32(stage, momeq, yn[e], acc + e, dt);
}

// ---- diffusion and hyperdiffusion (diffusion_ed, swm_operators.f90:855-975)
// coefdiv = K div x at the cells (blocks [0, nbc)), coefvort = K_tr zeta(x)
// at the triangles (the blocks after), with the folded FP32 coefficients of
// div_hx and rel_vort_tr
__global__ void __launch_bounds__(256) k_difcv32(DevMesh M, const float *__restrict__ x,
                                                 const float *__restrict__ kcv,
                                                 const float *__restrict__ kt,
                                                 float *__restrict__ coefdiv,
                                                 float *__restrict__ coefvort, int nbc) {
  if (static_cast<int>(blockIdx.x) < nbc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nv = M.nv;
    if (i >= nv) return;
    const int n = M.c_nnb[i];
    float d = 0.0f;
    for (int j = 0; j < n; ++j) d += x[__ldg(&M.c_ed[j * nv + i])] * __ldg(&M.c_div32[j * nv + i]);
    coefdiv[i] = kcv[i] * d;
  } else {
    const int t = (blockIdx.x - nbc) * blockDim.x + threadIdx.x;
    if (t >= M.nt) return;
    const int4 a = __ldg(&M.t_recA[t]), b = __ldg(&M.t_recB[t]);
    const float4 c = __ldg(&M.t_recC[t]);
    float z = __int_as_float(b.z) * x[a.x];
    z += __int_as_float(b.w) * x[a.y];
    z += c.x * x[a.z];
    coefvort[t] = __ldg(&kt[t]) * z;
  }
}

// lap = grad_ed(coefdiv) - grad_ed_tg(coefvort)
__global__ void __launch_bounds__(256) k_diflap32(DevMesh M, const float *__restrict__ coefdiv,
                                                  const float *__restrict__ coefvort,
                                                  float *__restrict__ lap) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne;
  if (e >= ne) return;
  const float g = (coefdiv[__ldg(&M.e_v[ne + e])] - coefdiv[__ldg(&M.e_v[e])]) *
                  __ldg(&M.e_grad32[e]);
  const float gt = (coefvort[__ldg(&M.e_sh[ne + e])] - coefvort[__ldg(&M.e_sh[e])]) *
                   __ldg(&M.e_gtg32[e]);
  lap[e] = g - gt;
}

// ---- cell-centred TRSK (variant 1), bodies in swm_k32_body.cuh ------------
// kEdgePV: q_tr is the edges' PV from the edge pre-pass (APVM); kZ false:
// no PV-flux terms (dtred forms its PV flux at the triangles)
template <bool kEdgePV, bool kZ = true>
__global__ void __launch_bounds__(512) k_cell32v2(DevMesh M, const float *__restrict__ hd,
                                                  const float *__restrict__ u,
                                                  const float *__restrict__ q_tr,
                                                  float *__restrict__ bern,
                                                  float *__restrict__ zflux,
                                                  const float *__restrict__ yn,
                                                  float *__restrict__ acc,
                                                  float *__restrict__ yout,
                                                  float *__restrict__ tend, int stage, float dt,
                                                  float grav, float h_ref,
                                                  const float *__restrict__ kcv,
                                                  float *__restrict__ coefdiv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.nv) return;
  cell_body<OneRun, LdPlain, kEdgePV, kZ>(M, i, OneRun{}, hd, u, q_tr, bern, zflux, yn, acc,
                                          yout, tend, stage, dt, grav, h_ref, kcv, coefdiv);
}

// ---- pxt16 in the cell-centred form (variants 1, 2) ------------------------
// The pass of k_cell32v2 with pxt16's pieces: each slot's edge PV from the
// edge pre-pass (the distance-weighted q_e of scalar_tr2ed's bary branch,
// APVM's upwinding when on), the Perot kinetic energy (kinetic_energy_hx,
// perhx branch: half the squared Perot velocity of the cell on its tangent
// plane) and pered's coefficients by cell in place of TRSK's kite fractions:
//     Z_c(i) = sum_{j != i} C_c(i, j) F_j (q_i + q_j)
// (coriolis_ed's pered branch, swm_operators.f90:1330-1377, split by cell).
// kEdgePV: the edges' PV from the edge pre-pass (APVM on); otherwise the
// cell forms pxt16's q_e from its triangles with the slot weights (c_qw32)
template <bool kEdgePV>
__global__ void __launch_bounds__(512) k_cell32p(DevMesh M, const float *__restrict__ hd,
                                                 const float *__restrict__ u,
                                                 const float *__restrict__ q_ed,
                                                 float *__restrict__ bern,
                                                 float *__restrict__ zflux,
                                                 const float *__restrict__ yn,
                                                 float *__restrict__ acc,
                                                 float *__restrict__ yout,
                                                 float *__restrict__ tend, int stage, float dt,
                                                 float grav, float h_ref,
                                                 const float *__restrict__ kcv,
                                                 float *__restrict__ coefdiv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  const int n = static_cast<int>(__ldg(&M.c_meta[i]) & 7u);
  int ed[6], nb[6], tr[6];
  float2 kd[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int4 pk = __ldg(&M.c_pk[j * nv + i]);
    kd[j] = __ldg(&M.c_kd[j * nv + i]);
    ed[j] = pk.x;
    nb[j] = pk.y;
    tr[j] = pk.z;
  }
  const float hi = hd[i], bt = __ldg(&M.c_bt32[i]), inva = __ldg(&M.c_inva32[i]);
  const float ynv = stage >= 0 ? yn[i] : 0.0f, accv = stage >= 1 ? acc[i] : 0.0f;
  float ue[6], hn[6], qs[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    ue[j] = u[ed[j]];
    hn[j] = hd[nb[j]];
    // q_tr here is the triangles' PV (kEdgePV false) or the edges' (true)
    qs[j] = q_ed[kEdgePV ? ed[j] : tr[j]];
  }
  if (!kEdgePV) {
    // scalar_tr2ed's bary branch: slot j's edge between triangles j-1, j
    float qt[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) qt[j] = qs[j];
    const float qlast = n == 6 ? qt[5] : qt[4];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      qs[j] = __ldg(&M.c_qw32[(2 * j) * nv + i]) * (j == 0 ? qlast : qt[j - 1]) +
              __ldg(&M.c_qw32[(2 * j + 1) * nv + i]) * qt[j];
  }
  // unused pentagon slots repeat slot 0 with zero weights (c_kd, c_apw32)
  float F[6], div = 0.0f, du = 0.0f, v[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    F[j] = ue[j] * (h_ref + 0.5f * (hi + hn[j]));
    div += F[j] * kd[j].y;
    du += ue[j] * kd[j].y;
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = fmaf(ue[j], __ldg(&M.c_apw32[(3 * j + c) * nv + i]), v[c]);
  }
  const float p0 = __ldg(&M.c_p32[i]), p1 = __ldg(&M.c_p32[nv + i]), p2 = __ldg(&M.c_p32[2 * nv + i]);
  const float vp = v[0] * p0 + v[1] * p1 + v[2] * p2;
  const float a0 = v[0] - vp * p0, a1 = v[1] - vp * p1, a2 = v[2] - vp * p2;
  const float ke = 0.5f * (a0 * a0 + a1 * a1 + a2 * a2);
  if (coefdiv) coefdiv[i] = kcv[i] * (du * inva);
  bern[i] = grav * (hi + bt) + ke;
#pragma unroll
  for (int si = 0; si < 6; ++si) {
    if (si >= n) break;
    float z = 0.0f;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j == si || j >= n) continue;
      z += __ldg(&M.c_C32[(6 * si + j) * nv + i]) * F[j] * (qs[si] + qs[j]);
    }
    zflux[6 * i + si] = z;
  }
  const float masseq = -div * inva;
  if (stage < 0) {
    tend[i] = masseq;
  } else {
    float a = accv;
    yout[i] = rk_stage32(stage, masseq, ynv, &a, dt);
    if (stage < 3) acc[i] = a;
  }
}

// ---- gass18 in the cell-centred form (variants 1, 2) ------------------------
// TRSK's weights and kinetic energy with gass18's PV: each slot's edge PV
// from the edge pre-pass (the rhombus PV of scalar_tr2ed's gass branch) and,
// in the pair (i, j) of coriolis_ed's gass branch (swm_operators.f90:
// 1378-1414), twice the PV of the connecting edge in place of q_i + q_j:
// the outer edge of the triangle shared by adjacent edges (c_gout), the
// cell edge between edges two apart, none for opposite edges (the layout
// checks this rule against edge_connection for every pair of every cell).
template <int N>
__device__ __forceinline__ void gass_cell(const float (&G)[6], const float (&qs)[6],
                                          const float (&qo)[6], const float (&R)[6],
                                          unsigned tneg, float (&Z)[6]) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
    float w = 0.0f, acc = 0.0f;
#pragma unroll
    for (int s = 1; s < N; ++s) {
      const int j = (i + s) % N;
      w += R[(i + s - 1) % N];
      float P;
      if (s == 1)
        P = 2.0f * qo[i];
      else if (s == N - 1)
        P = 2.0f * qo[j];
      else if (s == 2)
        P = 2.0f * qs[(i + 1) % N];
      else if (s == N - 2)
        P = 2.0f * qs[(i + N - 1) % N];
      else
        P = qs[i] + qs[j];
      acc += (w - 0.5f) * G[j] * P;
    }
    const float z = 0.5f * acc;
    Z[i] = ((tneg >> i) & 1u) ? -z : z;
  }
}

__global__ void __launch_bounds__(512) k_cell32g(DevMesh M, const float *__restrict__ hd,
                                                 const float *__restrict__ u,
                                                 const float *__restrict__ q_ed,
                                                 float *__restrict__ bern,
                                                 float *__restrict__ zflux,
                                                 const float *__restrict__ yn,
                                                 float *__restrict__ acc,
                                                 float *__restrict__ yout,
                                                 float *__restrict__ tend, int stage, float dt,
                                                 float grav, float h_ref,
                                                 const float *__restrict__ kcv,
                                                 float *__restrict__ coefdiv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nv = M.nv;
  if (i >= nv) return;
  const uint32_t meta = __ldg(&M.c_meta[i]);
  const int n = static_cast<int>(meta & 7u);
  const unsigned tneg = meta >> 8;
  int ed[6], nb[6], og[6];
  float R[6];
  float2 kd[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int4 pk = __ldg(&M.c_pk[j * nv + i]);
    kd[j] = __ldg(&M.c_kd[j * nv + i]);
    ed[j] = pk.x;
    nb[j] = pk.y;
    R[j] = __int_as_float(pk.w);
    og[j] = __ldg(&M.c_gout[j * nv + i]);
  }
  const float hi = hd[i], bt = __ldg(&M.c_bt32[i]), inva = __ldg(&M.c_inva32[i]);
  const float ynv = stage >= 0 ? yn[i] : 0.0f, accv = stage >= 1 ? acc[i] : 0.0f;
  float ue[6], hn[6], qs[6], qo[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    ue[j] = u[ed[j]];
    hn[j] = hd[nb[j]];
    qs[j] = q_ed[ed[j]];
    qo[j] = q_ed[og[j]];
  }
  float G[6], div = 0.0f, ke = 0.0f, du = 0.0f;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float F = ue[j] * (h_ref + 0.5f * (hi + hn[j]));
    G[j] = F * kd[j].y;
    div += G[j];
    ke += kd[j].x * (ue[j] * ue[j]);
    du += ue[j] * kd[j].y;
  }
  if (coefdiv) coefdiv[i] = kcv[i] * (du * inva);
  bern[i] = grav * (hi + bt) + ke;
  // the layout admits this kernel only on pentagons and hexagons
  float Z[6];
  if (n == 6)
    gass_cell<6>(G, qs, qo, R, tneg, Z);
  else
    gass_cell<5>(G, qs, qo, R, tneg, Z);
#pragma unroll
  for (int j = 0; j < 6; ++j)
    if (j < n) zflux[6 * i + j] = Z[j];
  const float masseq = -div * inva;
  if (stage < 0) {
    tend[i] = masseq;
  } else {
    float a = accv;
    yout[i] = rk_stage32(stage, masseq, ynv, &a, dt);
    if (stage < 3) acc[i] = a;
  }
}

// ---- dtred in the cell-centred form (variants 1, 2) ------------------------
// coriolis_ed's dtred branch (swm_operators.f90:1310-1329) reconstructs q F
// at the edge's two triangles: Q_e = -sum_i w_i q_ti (P_ti . nr_e), P_t the
// Perot vector of uh over the triangle's edges.  The triangle kernel forms
// q_t P_t once per triangle (uh_s = u_s (h_ref + the mean of the two
// corners on edge s), the edge pre-pass's F bit for bit); the edge kernel
// projects the two triangles' vectors on its normal.
__global__ void __launch_bounds__(512) k_tri32d(DevMesh M, const float *__restrict__ hd,
                                                const float *__restrict__ u,
                                                float *__restrict__ q_tr, float h_ref,
                                                int pv_on, int *flags,
                                                const float *__restrict__ kt,
                                                float *__restrict__ coefvort,
                                                float *__restrict__ wq) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.nt;
  if (t >= nt) return;
  const int4 a = __ldg(&M.t_recA[t]), b = __ldg(&M.t_recB[t]);
  const float4 c = __ldg(&M.t_recC[t]);
  const int ed[3] = {a.x, a.y, a.z}, cv[3] = {a.w, b.x, b.y};
  const float circ[3] = {__int_as_float(b.z), __int_as_float(b.w), c.x};
  const float kite[3] = {c.y, c.z, c.w};
  tri_core<OneRun, LdPlain>(t, OneRun{}, ed, cv, circ, kite, __ldg(&M.t_f32[t]), hd, u, q_tr,
                            h_ref, pv_on, flags, kt, coefvort, nullptr);
  const float q = q_tr[t];
  const unsigned opp = __ldg(&M.t_dopp[t]);
  const float hc[3] = {hd[cv[0]], hd[cv[1]], hd[cv[2]]};
  float P[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const int o = static_cast<int>((opp >> (2 * s)) & 3u);
    const float ha = o == 0 ? hc[1] : hc[0], hb = o == 2 ? hc[1] : hc[2];
    const float uh = u[ed[s]] * (h_ref + 0.5f * (ha + hb));
#pragma unroll
    for (int k = 0; k < 3; ++k) P[k] = fmaf(uh, __ldg(&M.t_dpa32[(3 * s + k) * nt + t]), P[k]);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) wq[k * nt + t] = q * P[k];
}

// -grad B - Q_e and the momentum RK stage of edge e (dtred)
__global__ void __launch_bounds__(512) k_edge32d(DevMesh M, const float *__restrict__ bern,
                                                 const float *__restrict__ wq,
                                                 const float *__restrict__ yn,
                                                 float *__restrict__ acc,
                                                 float *__restrict__ yout,
                                                 float *__restrict__ tend, int stage, float dt,
                                                 int mom_on, const float *__restrict__ dif1,
                                                 const float *__restrict__ dif2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = M.ne, nt = M.nt;
  if (e >= ne) return;
  const float g = (bern[__ldg(&M.e_v[ne + e])] - bern[__ldg(&M.e_v[e])]) * __ldg(&M.e_grad32[e]);
  const float n0 = __ldg(&M.e_nr32[e]), n1 = __ldg(&M.e_nr32[ne + e]), n2 = __ldg(&M.e_nr32[2 * ne + e]);
  float q = 0.0f;
#pragma unroll
  for (int si = 0; si < 2; ++si) {
    const int t = __ldg(&M.e_sh[si * ne + e]);
    const float d = wq[t] * n0 + wq[nt + t] * n1 + wq[2 * nt + t] * n2;
    q -= __ldg(&M.e_dw32[si * ne + e]) * d;
  }
  float momeq = -g - q;
  if (dif1) momeq += dif1[e];
  if (dif2) momeq -= dif2[e];
  if (!mom_on) momeq = 0.0f;
  if (stage < 0)
    tend[e] = momeq;
  else
    yout[e] = rk_stage32(stage, momeq, yn[e], acc + e, dt);
}

// ---- variant 2: the triangle kernel on records with 16-bit indices -------
__global__ void __launch_bounds__(512) k_tri32c(DevMesh M, const float *__restrict__ hd,
                                                const float *__restrict__ u,
                                                float *__restrict__ q_tr, float h_ref,
                                                int pv_on, int *flags,
                                                const float *__restrict__ kt,
                                                float *__restrict__ coefvort) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.nt) return;
  tri_body16(M, t, hd, u, q_tr, h_ref, pv_on, flags, kt, coefvort);
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
                                                  const float *__restrict__ corr,
                                                  const float *__restrict__ dif1,
                                                  const float *__restrict__ dif2) {
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
    // diffusion, then hyperdiffusion
    if (dif1) {
      const float2 d = reinterpret_cast<const float2 *>(dif1)[p];
      m0 += d.x;
      m1 += d.y;
    }
    if (dif2) {
      const float2 d = reinterpret_cast<const float2 *>(dif2)[p];
      m0 -= d.x;
      m1 -= d.y;
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
              mom_on, erad, corr, dif1, dif2);
  }
}

// the error proxy's sums (launch_departure): grid-stride over the edges,
// warp shuffles, one pair of FP64 partial sums per block
__global__ void __launch_bounds__(256) k_departure(DevMesh M, const float *__restrict__ a,
                                                   const float *__restrict__ b,
                                                   const float *__restrict__ c,
                                                   double *__restrict__ part) {
  __shared__ double sd[8], sb[8];
  double d2 = 0.0, b2 = 0.0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < M.ne; e += gridDim.x * blockDim.x) {
    const double w = __ldg(&M.e_area32[e]), bb = b[e];
    const double dd = static_cast<double>(a[e]) - bb, rr = bb - static_cast<double>(c[e]);
    d2 += w * dd * dd;
    b2 += w * rr * rr;
  }
  for (int o = 16; o > 0; o >>= 1) {
    d2 += __shfl_down_sync(0xffffffffu, d2, o);
    b2 += __shfl_down_sync(0xffffffffu, b2, o);
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sd[wid] = d2;
    sb[wid] = b2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int k = 0; k < 8; ++k) {
      x += sd[k];
      y += sb[k];
    }
    part[2 * blockIdx.x] = x;
    part[2 * blockIdx.x + 1] = y;
  }
}

inline int nblocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void launch_departure(const DevMesh &M, const float *a, const float *b, const float *c,
                      double *part, int nblk, cudaStream_t s) {
  k_departure<<<nblk, 256, 0, s>>>(M, a, b, c, part);
}

void launch_stage32(const DevMesh &M, const Work<float> &W, const float *h_in,
                    const float *u_in, float *h_out, float *u_out, int stage, float dt,
                    cudaStream_t s, cudaEvent_t *ev) {
  const Tune &T = W.tune;
  const float grav = static_cast<float>(M.grav);
  if (ev) cudaEventRecord(ev[0], s);
  const Diffusion<float> &D = W.dif;
  const float *dif1 = D.k2 ? D.lap : nullptr, *dif2 = D.k4 ? D.lap2 : nullptr;
  const int nbc = nblocks(M.nv, 256), nbt = nblocks(M.nt, 256);
  // the edge gradients of the diffusion (and the second application of
  // hyperdiffusion) once K div u and K_tr zeta are written
  auto diffusion_tail = [&]() {
    if (!D.on) return;
    k_diflap32<<<nblocks(M.ne, 256), 256, 0, s>>>(M, D.coefdiv, D.coefvort, D.lap);
    if (D.k4) {
      k_difcv32<<<nbc + nbt, 256, 0, s>>>(M, D.lap, D.kcv, D.kt, D.coefdiv, D.coefvort, nbc);
      k_diflap32<<<nblocks(M.ne, 256), 256, 0, s>>>(M, D.coefdiv, D.coefvort, D.lap2);
    }
  };
  if (T.variant == 0 && D.on)  // variant 0: K div u and K_tr zeta in their own pass
    k_difcv32<<<nbc + nbt, 256, 0, s>>>(M, u_in, D.kcv, D.kt, D.coefdiv, D.coefvort, nbc);
  float *cvort = (T.variant >= 1 && D.on) ? D.coefvort : nullptr;
  const bool dtred1 = T.variant >= 1 && W.scheme == IMODEL_SWM_DTRED;
  // gass18 needs the triangle depths of the 32-bit triangle kernel, dtred
  // the Perot vectors of its own
  if (dtred1)
    k_tri32d<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ref,
                                                           W.pv_on, W.flags, D.kt, cvort, W.vhq);
  else if (T.variant == 2 && W.scheme != IMODEL_SWM_GASS18)
    k_tri32c<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(M, h_in, u_in, W.q_tr, W.h_ref,
                                                           W.pv_on, W.flags, D.kt, cvort);
  else
    k_tri32<<<nblocks(M.nt, T.bs_tri), T.bs_tri, 0, s>>>(
        M, h_in, u_in, W.q_tr, W.h_ref, W.pv_on, W.flags, D.kt, cvort,
        W.scheme == IMODEL_SWM_GASS18 ? W.h_trs : nullptr);
  if (T.variant >= 1) {
    if (ev) cudaEventRecord(ev[1], s);
    // learned correction: formed once per step from the first stage's state
    if (W.learned && stage <= 0)
      learned_launch(M, *W.learned, h_in, u_in, W.q_tr, W.h_ref, T.mlp_gather, W.flags, s);
    const Apvm<float> &A = W.apvm;
    const bool pxt = W.scheme == IMODEL_SWM_PXT16, gass = W.scheme == IMODEL_SWM_GASS18;
    // APVM (swm_operators.f90:1495-1502) and pxt16's distance-weighted q_e:
    // the PV of every edge from the edge pre-pass, read by the cells in
    // place of the triangle average
    if (A.on)
      k_apvm32<<<nbt + nblocks(M.nv, 256), 256, 0, s>>>(M, W.q_tr, u_in, A.qg, A.vhx, nbt);
    if (A.on || gass)
      k_edge_pre32<<<nblocks(M.ne, T.bs_pre), T.bs_pre, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.h_ed, W.uh, W.q_ed, W.h_ref, A.on ? A.qg : nullptr, A.vhx,
          A.coef, pxt || gass ? M.e_qw32 : nullptr, gass ? W.h_trs : nullptr, W.pv_on, W.flags);
    if (ev) cudaEventRecord(ev[2], s);
    if (gass)
      k_cell32g<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_ed, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    else if (pxt && A.on)
      k_cell32p<true><<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_ed, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    else if (pxt)
      k_cell32p<false><<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    else if (dtred1)
      k_cell32v2<false, false><<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    else if (A.on)
      k_cell32v2<true><<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_ed, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    else
      k_cell32v2<false><<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(
          M, h_in, u_in, W.q_tr, W.bern, W.zflux, W.yn_h, W.acc_h, h_out, W.tend_h, stage, dt,
          grav, W.h_ref, D.kcv, D.on ? D.coefdiv : nullptr);
    diffusion_tail();
    if (ev) cudaEventRecord(ev[3], s);
    if (dtred1)
      k_edge32d<<<nblocks(M.ne, T.bs_edge), T.bs_edge, 0, s>>>(
          M, W.bern, W.vhq, W.yn_u, W.acc_u, u_out, W.tend_u, stage, dt, W.mom_on, dif1, dif2);
    else
      k_edge32v2<<<nblocks((M.ne + 1) / 2, T.bs_edge), T.bs_edge, 0, s>>>(
          M, W.bern, W.zflux, W.yn_u, W.acc_u, u_out, W.tend_u, stage, dt, W.mom_on,
          static_cast<float>(M.erad), W.learned ? W.learned->corr : nullptr, dif1, dif2);
    if (ev) cudaEventRecord(ev[4], s);
    return;
  }
  if (ev) cudaEventRecord(ev[1], s);
  const Apvm<float> &A = W.apvm;
  if (A.on) {
    const int nbt = nblocks(M.nt, 256);
    k_apvm32<<<nbt + nblocks(M.nv, 256), 256, 0, s>>>(M, W.q_tr, u_in, A.qg, A.vhx, nbt);
  }
  // the method wrappers (variant 0 only): pxt16 (distance-weighted q_e,
  // Perot KE, pered), gass18 (rhombus PV, connecting-edge PV), dtred
  const int sch = W.scheme;
  const bool pxt = sch == IMODEL_SWM_PXT16, gass = sch == IMODEL_SWM_GASS18;
  k_edge_pre32<<<nblocks(M.ne, T.bs_pre), T.bs_pre, 0, s>>>(
      M, h_in, u_in, W.q_tr, W.h_ed, W.uh, W.q_ed, W.h_ref, A.on ? A.qg : nullptr, A.vhx, A.coef,
      pxt || gass ? M.e_qw32 : nullptr, gass ? W.h_trs : nullptr, W.pv_on, W.flags);
  if (ev) cudaEventRecord(ev[2], s);
  k_cell32<<<nblocks(M.nv, T.bs_cell), T.bs_cell, 0, s>>>(M, h_in, u_in, W.uh, W.bern, W.yn_h,
                                                           W.acc_h, h_out, W.tend_h, stage, dt,
                                                           grav, pxt ? 1 : 0);
  diffusion_tail();
  if (ev) cudaEventRecord(ev[3], s);
  k_edge32<<<nblocks(M.ne, T.bs_edge), T.bs_edge, 0, s>>>(
      M, W.bern, W.uh, W.q_ed, W.yn_u, W.acc_u, u_out, W.tend_u, stage, dt, W.mom_on, dif1, dif2,
      gass ? M.e_stq : nullptr, W.q_tr, sch == IMODEL_SWM_DTRED ? 1 : 0);
  if (ev) cudaEventRecord(ev[4], s);
}

}  // namespace imodel
