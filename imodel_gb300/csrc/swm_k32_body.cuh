// Per-entity bodies of the FP32 cell-centred TRSK stage (internal header).
//
// Shared by the single-run kernels (swm_k32.cu) and the ensemble kernel
// (swm_ens.cu).  The index policy maps an entity to its slot in a state
// array: one run stores entity i at i, an ensemble stores member m of entity
// i at i*M + m (members fastest), so that the threads of a warp that share
// an entity read its geometry once and the members' values contiguously.
#pragma once
#include "swm_common.cuh"

namespace imodel {

struct OneRun {
  __device__ __forceinline__ int operator()(int i) const { return i; }
};
struct Member {
  int M, m;
  __device__ __forceinline__ int operator()(int i) const { return i * M + m; }
};

// Loads of fields that change during a run.  Separate launches see each
// other's writes, so plain loads are fine there; inside the persistent
// ensemble kernel another block may have rewritten the value since this SM
// cached it, so those loads go through L2 (ld.global.cg), never through the
// incoherent L1 / read-only path.
struct LdPlain {
  static __device__ __forceinline__ float ld(const float *p) { return *p; }
};
struct LdL2 {
  static __device__ __forceinline__ float ld(const float *p) { return __ldcg(p); }
};

// ode_rk4 stage update (swm.f90:2647-2678) in FP32
__device__ __forceinline__ float rk_stage32(int stage, float k, float yn, float *acc, float dt) {
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
// from a triangle's decoded record: edges, cells, circulation and kite
// coefficients, Coriolis parameter; the sums run in slot order 0, 1, 2
template <class Ix, class Ld>
__device__ __forceinline__ void tri_core(int t, Ix ix, const int (&ed)[3], const int (&cv)[3],
                                         const float (&circ)[3], const float (&kite)[3],
                                         float f, const float *__restrict__ hd,
                                         const float *__restrict__ u, float *__restrict__ q_tr,
                                         float h_ref, int pv_on, int *flags,
                                         const float *__restrict__ kt = nullptr,
                                         float *__restrict__ coefvort = nullptr,
                                         float *__restrict__ ht_out = nullptr) {
  float eta = f;
  float ht = 0.0f, z = 0.0f;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    const float us = Ld::ld(u + ix(ed[s]));
    eta += circ[s] * us;
    z += circ[s] * us;
    ht += kite[s] * Ld::ld(hd + ix(cv[s]));
  }
  // with diffusion on: K_tr times the relative vorticity
  if (coefvort) coefvort[ix(t)] = kt[t] * z;
  ht += h_ref;
  // gass18: the depth at the triangle for the rhombus PV of the edges
  if (ht_out) ht_out[ix(t)] = ht;
  float q = 0.0f;
  if (pv_on) {
    // scalar_elem_divide guard, swm_operators.f90:1604-1606
    if (fabsf(ht) < 1.1920928955078125e-12f)
      atomicOr(flags, 1);
    else
      q = eta / ht;
  }
  q_tr[ix(t)] = q;
}

template <class Ix, class Ld = LdPlain>
__device__ __forceinline__ void tri_body(const DevMesh &M, int t, Ix ix,
                                         const float *__restrict__ hd,
                                         const float *__restrict__ u, float *__restrict__ q_tr,
                                         float h_ref, int pv_on, int *flags,
                                         const float *__restrict__ kt = nullptr,
                                         float *__restrict__ coefvort = nullptr,
                                         float *__restrict__ ht_out = nullptr) {
  // three 16-byte records instead of 12 scalar streams (fewer load
  // instructions in flight per SM)
  const int4 a = __ldg(&M.t_recA[t]), b = __ldg(&M.t_recB[t]);
  const float4 c = __ldg(&M.t_recC[t]);
  const int ed[3] = {a.x, a.y, a.z}, cv[3] = {a.w, b.x, b.y};
  const float circ[3] = {__int_as_float(b.z), __int_as_float(b.w), c.x};
  const float kite[3] = {c.y, c.z, c.w};
  tri_core<Ix, Ld>(t, ix, ed, cv, circ, kite, __ldg(&M.t_f32[t]), hd, u, q_tr, h_ref, pv_on,
                   flags, kt, coefvort, ht_out);
}

// the same from 40-byte records with 16-bit indices (single runs): a warp of
// 32 triangles shares one base per index kind (t_wb); a warp whose indices
// span more than 65,536 takes its indices from the 32-bit records instead
// (warp-uniform branch).  The records and the bases are loaded together, so
// that the gathers wait for one round trip, as with the 32-bit records.
__device__ __forceinline__ void tri_body16(const DevMesh &M, int t, const float *__restrict__ hd,
                                           const float *__restrict__ u,
                                           float *__restrict__ q_tr, float h_ref, int pv_on,
                                           int *flags, const float *__restrict__ kt,
                                           float *__restrict__ coefvort) {
  const int2 wb = __ldg(&M.t_wb[t >> 5]);
  const uint4 a = __ldg(&M.t_c16A[t]);
  const float4 b = __ldg(&M.t_c16B[t]);
  const float2 c = __ldg(&M.t_c16C[t]);
  int ed[3], cv[3];
  if (wb.y >= 0) {
    ed[0] = wb.x + static_cast<int>(a.x & 0xFFFFu);
    ed[1] = wb.x + static_cast<int>(a.x >> 16);
    ed[2] = wb.x + static_cast<int>(a.y & 0xFFFFu);
    cv[0] = wb.y + static_cast<int>(a.y >> 16);
    cv[1] = wb.y + static_cast<int>(a.z & 0xFFFFu);
    cv[2] = wb.y + static_cast<int>(a.z >> 16);
  } else {
    const int4 ra = __ldg(&M.t_recA[t]), rb = __ldg(&M.t_recB[t]);
    ed[0] = ra.x;
    ed[1] = ra.y;
    ed[2] = ra.z;
    cv[0] = ra.w;
    cv[1] = rb.x;
    cv[2] = rb.y;
  }
  const float circ[3] = {__uint_as_float(a.w), b.x, b.y};
  const float kite[3] = {b.z, b.w, c.x};
  tri_core<OneRun, LdPlain>(t, OneRun{}, ed, cv, circ, kite, c.y, hd, u, q_tr, h_ref, pv_on,
                            flags, kt, coefvort);
}

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

// the arithmetic of one cell from its gathered values: div F, K, the
// Bernoulli potential, the PV-flux contributions Z (cell-major zflux) and
// the mass RK stage.  kEdgePV: qt holds the PV of the cell's edges (formed
// by the edge pre-pass, APVM's upwinding included) instead of the PV of its
// triangles.
template <class Ix = OneRun, bool kEdgePV = false, bool kZ = true>
__device__ __forceinline__ void cell_math(int i, uint32_t meta, const float (&R)[6],
                                          const float2 (&kd)[6], const float (&ue)[6],
                                          const float (&hn)[6], const float (&qt)[6], float hi,
                                          float bt, float inva, float ynv, float accv,
                                          float *__restrict__ bern, float *__restrict__ zflux,
                                          float *__restrict__ acc, float *__restrict__ yout,
                                          float *__restrict__ tend, int stage, float dt,
                                          float grav, float h_ref, Ix ix = Ix{},
                                          const float *__restrict__ kcv = nullptr,
                                          float *__restrict__ coefdiv = nullptr) {
  const int n = static_cast<int>(meta & 7u);
  const unsigned tneg = meta >> 8;
  float G[6], qs[6];
  float div = 0.0f, ke = 0.0f, du = 0.0f;
  const float qlast = n == 6 ? qt[5] : (n == 5 ? qt[4] : (n == 4 ? qt[3] : qt[2]));
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    // F_e = u_e h_e, h_e the two-cell average (scalar_hx2ed)
    const float F = ue[j] * (h_ref + 0.5f * (hi + hn[j]));
    G[j] = F * kd[j].y;
    // q_e: edge j lies between triangles j-1 and j (scalar_tr2ed)
    qs[j] = kEdgePV ? qt[j] : 0.5f * ((j == 0 ? qlast : qt[j - 1]) + qt[j]);
    div += G[j];
    ke += kd[j].x * (ue[j] * ue[j]);
    du += ue[j] * kd[j].y;
  }
  // with diffusion on: K times the divergence of u
  if (coefdiv) coefdiv[ix(i)] = kcv[ix(i)] * (du * inva);
  bern[ix(i)] = grav * (hi + bt) + ke;
  // kZ false (dtred): the edges form their PV flux from the triangles
  if (kZ) {
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
      if (j < n) zflux[ix(6 * i + j)] = Z[j];
  }
  const float masseq = -div * inva;
  if (stage < 0) {
    tend[ix(i)] = masseq;
  } else {
    float a = accv;
    yout[ix(i)] = rk_stage32(stage, masseq, ynv, &a, dt);
    if (stage < 3) acc[ix(i)] = a;
  }
}

// div F, K, Bernoulli potential, PV-flux contributions Z (cell-major
// zflux[cell][6]) and the mass RK stage of cell i, from its decoded slot
// records: edge, neighbour, triangle, kite fraction R and {KE weight,
// ttgout*d} of each slot (unused pentagon slots repeat slot 0 with zero
// weights), gathering its neighbours' values.  The cell's own values come in
// as arguments: h (deviation) hi, b bt, 1/(A a) inva, y_n ynv and the RK
// accumulator accv (read for stages 1-3).
template <class Ix, class Ld, bool kEdgePV = false, bool kZ = true>
__device__ __forceinline__ void cell_core(int i, Ix ix, uint32_t meta,
                                          const int (&ed)[6], const int (&nb)[6],
                                          const int (&tr)[6], const float (&R)[6],
                                          const float2 (&kd)[6], float hi, float bt, float inva,
                                          float ynv, float accv, const float *__restrict__ hd,
                                          const float *__restrict__ u,
                                          const float *__restrict__ q_tr,
                                          float *__restrict__ bern, float *__restrict__ zflux,
                                          float *__restrict__ acc, float *__restrict__ yout,
                                          float *__restrict__ tend, int stage, float dt,
                                          float grav, float h_ref, const float *__restrict__ kcv = nullptr,
                                          float *__restrict__ coefdiv = nullptr) {
  float ue[6], hn[6], qt[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    ue[j] = Ld::ld(u + ix(ed[j]));
    hn[j] = Ld::ld(hd + ix(nb[j]));
    // kEdgePV: q_tr is the edges' PV, indexed by the slot's edge
    qt[j] = Ld::ld(q_tr + ix(kEdgePV ? ed[j] : tr[j]));
  }
  cell_math<Ix, kEdgePV, kZ>(i, meta, R, kd, ue, hn, qt, hi, bt, inva, ynv, accv, bern, zflux,
                             acc, yout, tend, stage, dt, grav, h_ref, ix, kcv, coefdiv);
}

// the cell's own values from global memory
template <class Ix, class Ld>
__device__ __forceinline__ void cell_own(const DevMesh &M, int i, Ix ix,
                                         const float *__restrict__ hd,
                                         const float *__restrict__ yn,
                                         const float *__restrict__ acc, int stage, float &hi,
                                         float &bt, float &inva, float &ynv, float &accv) {
  hi = Ld::ld(hd + ix(i));
  bt = __ldg(&M.c_bt32[i]);
  inva = __ldg(&M.c_inva32[i]);
  ynv = stage >= 0 ? Ld::ld(yn + ix(i)) : 0.0f;
  accv = stage >= 1 ? Ld::ld(acc + ix(i)) : 0.0f;
}

template <class Ix, class Ld = LdPlain, bool kEdgePV = false, bool kZ = true>
__device__ __forceinline__ void cell_body(const DevMesh &M, int i, Ix ix,
                                          const float *__restrict__ hd,
                                          const float *__restrict__ u,
                                          const float *__restrict__ q_tr,
                                          float *__restrict__ bern, float *__restrict__ zflux,
                                          const float *__restrict__ yn, float *__restrict__ acc,
                                          float *__restrict__ yout, float *__restrict__ tend,
                                          int stage, float dt, float grav, float h_ref,
                                          const float *__restrict__ kcv = nullptr,
                                          float *__restrict__ coefdiv = nullptr) {
  const int nv = M.nv;
  const uint32_t meta = __ldg(&M.c_meta[i]);
  int ed[6], nb[6], tr[6];
  float R[6];
  float2 kd[6];
  // all slot records first, so that every load is in flight before the
  // gathers
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int4 pk = __ldg(&M.c_pk[j * nv + i]);
    kd[j] = __ldg(&M.c_kd[j * nv + i]);
    ed[j] = pk.x;
    nb[j] = pk.y;
    tr[j] = pk.z;
    R[j] = __int_as_float(pk.w);
  }
  float hi, bt, inva, ynv, accv;
  cell_own<Ix, Ld>(M, i, ix, hd, yn, acc, stage, hi, bt, inva, ynv, accv);
  cell_core<Ix, Ld, kEdgePV, kZ>(i, ix, meta, ed, nb, tr, R, kd, hi, bt, inva, ynv, accv, hd, u,
                                 q_tr, bern, zflux, acc, yout, tend, stage, dt, grav, h_ref, kcv,
                                 coefdiv);
}

// -grad B - (Z_c1 + Z_c2) / l_e and the momentum RK stage of edge e
template <class Ix, class Ld = LdPlain>
__device__ __forceinline__ void edge_body(const DevMesh &M, int e, Ix ix, uint2 w,
                                          const float *__restrict__ bern,
                                          const float *__restrict__ zflux,
                                          const float *__restrict__ yn, float *__restrict__ acc,
                                          float *__restrict__ yout, float *__restrict__ tend,
                                          int stage, float dt, int mom_on, float erad,
                                          const float *__restrict__ corr = nullptr,
                                          const float *__restrict__ dif1 = nullptr,
                                          const float *__restrict__ dif2 = nullptr) {
  const int c1 = static_cast<int>(w.x & 0x0FFFFFFFu), c2 = static_cast<int>(w.y & 0x0FFFFFFFu);
  const int s1 = static_cast<int>(w.x >> 28), s2 = static_cast<int>(w.y >> 28);
  const float g = __ldg(&M.e_grad32[e]);  // 1 / (l_e a)
  const float grad = (Ld::ld(bern + ix(c2)) - Ld::ld(bern + ix(c1))) * g;
  const float q = (Ld::ld(zflux + ix(6 * c1 + s1)) + Ld::ld(zflux + ix(6 * c2 + s2))) * (g * erad);
  float momeq = -grad - q;
  // learned correction of the PV flux (frozen over the RK step)
  if (corr) momeq += corr[ix(e)];
  // diffusion, then hyperdiffusion
  if (dif1) momeq += dif1[ix(e)];
  if (dif2) momeq -= dif2[ix(e)];
  if (!mom_on) momeq = 0.0f;
  if (stage < 0)
    tend[ix(e)] = momeq;
  else
    yout[ix(e)] = rk_stage32(stage, momeq, Ld::ld(yn + ix(e)), acc + ix(e), dt);
}

}  // namespace imodel
