// Device data layout of the TRSK shallow-water step (internal header).
//
// Cells are renumbered along a 3-D Hilbert curve through their positions on
// the sphere; edges are renumbered by their lower-numbered cell and
// triangles by their lowest vertex, so that the entities one thread block
// touches sit in a few contiguous runs of HBM.  All per-entity lists are
// padded to a fixed width and stored slot-major (slot j of entity i at
// [j * n + i]) so that a warp reading slot j of 32 consecutive entities
// issues one coalesced request.
//
// Two coefficient sets are kept:
//  * FP64 "reference order": the factors the Fortran multiplies by, in the
//    Fortran's order, so the FP64 kernels reproduce the reference's
//    rounding step by step (sign factors +-1 are folded into a coefficient,
//    which is exact).
//  * FP32 "folded": every constant factor of a term folded into one
//    coefficient computed in FP64 and rounded once.
#pragma once
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "imodel_swm.h"

namespace imodel {

// An allocator whose resize() leaves new elements uninitialised: the layout
// builder writes every element of the arrays it resizes and fills the
// padded ones in parallel, so the serial zero-filling of a level-10 layout's
// ~15 GB is skipped.  assign(n, v) still fills.
template <class T>
struct HostAlloc : std::allocator<T> {
  using std::allocator<T>::allocator;
  template <class U>
  struct rebind {
    using other = HostAlloc<U>;
  };
  template <class U>
  void construct(U *p) noexcept {
    ::new (static_cast<void *>(p)) U;
  }
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
template <class T>
using HVec = std::vector<T, HostAlloc<T>>;

constexpr int kMaxNb = 6;     // cells have 5 or 6 edges on icosahedral grids
constexpr int kMaxSt = 10;    // TRSK stencil: nnb(c1) + nnb(c2) - 2 <= 10

struct Layout {
  int nv = 0, ne = 0, nt = 0;
  double erad = 0, grav = 0, omega = 0;

  // permutations (new index -> reference index, 0-based) and inverses
  HVec<int32_t> cell_n2o, cell_o2n, edge_n2o, edge_o2n, tri_n2o, tri_o2n;

  // cells, slot-major [kMaxNb][nv]
  HVec<int8_t> c_nnb;                 // [nv]
  HVec<int32_t> c_ed;                 // edge of slot j (-1 pad)
  HVec<double> c_sd;                  // ttgout * edhx%leng of slot j
  HVec<double> c_areag;               // [nv] hx%areag
  HVec<double> c_cellarea;            // [nv] sum_j 0.25*l*d (KE tiled area)
  HVec<double> c_bt;                  // [nv] bottom topography
  HVec<float> c_div32;                // ttgout*d/(A*erad)
  HVec<float> c_kew32;                // 0.25*l*d / cell_area
  // cell-centred TRSK variant (FP32): the PV flux of an edge is assembled
  // from the two cells' kite fractions instead of a 10-entry edge stencil
  HVec<int32_t> c_nb;                 // neighbour cell across slot j
  HVec<int32_t> c_tr;                 // triangle v%tr(j) (edges j, j+1)
  HVec<float> c_R32;                  // kite fraction hxtr_area(j)
  HVec<float> c_dg32;                 // ttgout(j) * edhx%leng(j)
  HVec<float> c_inva32;               // [nv] 1/(A*erad)
  HVec<uint32_t> c_meta;              // [nv] nnb | tnrccw<0 bits << 8
  HVec<uint32_t> e_vs;                // [2][ne] cell | slot << 28
  // the same per-slot data packed for 16-byte loads, slot-major [6][nv]:
  // {edge, neighbour, triangle, kite fraction bits} and {KE weight,
  // ttgout*d}; unused slots of pentagons repeat slot 0 with zero weights
  HVec<int32_t> c_pk;                 // [6][nv][4]
  HVec<float> c_kd;                   // [6][nv][2]
  HVec<uint32_t> e_vs2;               // [ne][2] both cell words of an edge

  // edges [ne] and [2][ne]
  HVec<int32_t> e_v;                  // [2][ne] cells (ed%v = edhx%sh)
  HVec<int32_t> e_sh;                 // [2][ne] triangles (ed%sh)
  HVec<double> e_leng;                // ed%leng
  HVec<double> e_dleng;               // edhx%leng
  HVec<double> e_kew;                 // 0.25*l*d (KE weight, FP64)
  HVec<float> e_grad32;               // 1/(l*erad)
  // grad_ed_tg (swm_operators.f90:738-777, HTC): sign of ed%nr . (c2 - c1)
  // for the circumcentres c1, c2 of ed%sh(1), ed%sh(2), and the FP32 factor
  // sign / (edhx%leng * erad); used by the (hyper)diffusion terms
  HVec<double> e_sgtg;
  HVec<float> e_gtg32;
  HVec<int8_t> e_nst;                 // stencil length
  HVec<int32_t> e_stk;                // [kMaxSt][ne] stencil edges
  HVec<double> e_stw;                 // [kMaxSt][ne] trskw * signcor
  HVec<float> e_stc32;                // [kMaxSt][ne] 0.5*w*s*d_k/l_e

  // triangles, slot-major [3][nt]
  HVec<int32_t> t_ed, t_v;
  HVec<double> t_lt;                  // ed%leng * tr%tg
  HVec<double> t_kite;                // tr%trhx_area
  HVec<double> t_areag;               // [nt]
  HVec<double> t_f;                   // [nt] 2*omega*sin(lat_c)
  // APVM points, [3][n] in device order, empty without ed%nr: ed%c%p, the
  // circumcentre direction of each triangle (circumcentre()), v%p
  HVec<double> e_c, t_c, c_p;
  // the FP32 step's APVM weights: per triangle slot s and component k,
  // t_apw32[(3s+k)][nt] = -tr%tg (ed%c%p - tr%c%p)_k ed%leng / tr%areag,
  // per cell slot j, c_apw32[(3j+k)][nv] = ttgout (ed%c%p - v%p)_k
  // edhx%leng / hx%areag (0 in a pentagon's sixth slot); the unit vectors
  // t_cc32 [3][nt] and c_p32 [3][nv] for the tangent-plane projections
  HVec<float> t_apw32, t_cc32, c_apw32, c_p32;
  // a triangle's FP32 stage inputs as three 16-byte records, [nt] each:
  //   A {edge 0, edge 1, edge 2, cell 0}  B {cell 1, cell 2, circ 0, circ 1}
  //   C {circ 2, kite 0, kite 1, kite 2}  (circ, kite: FP32 bit patterns)
  HVec<int32_t> t_recA, t_recB, t_recC;
  // the same with 16-bit indices against per-warp bases t_wb [nwarps][2] =
  // {edge, cell} (cell = -1: the warp keeps the 32-bit records):
  //   A {e0 | e1 << 16, e2 | c0 << 16, c1 | c2 << 16, circ 0}
  //   B {circ 1, circ 2, kite 0, kite 1}  C {kite 2, f}
  HVec<uint32_t> t_c16A;
  HVec<float> t_c16B, t_c16C;
  HVec<int32_t> t_wb;
  HVec<float> t_circ32;               // l*tg/(A*erad)
  HVec<float> t_kite32;               // kite/A
  HVec<float> t_f32;

  // per-edge reference-ordered weight for edge integrals: l*d*0.5
  HVec<double> e_area;

  // the geometry of the other method wrappers (FP64, device order; empty for
  // trsk10), as initialize_gridprop precomputes it (swm.f90:1005-1028):
  //   t_bary  [3][nt] tr%c%b, barycentric coordinates of the circumcentre
  //           (bar_coord_tr, smeshpack.f90:5200-5245; pxt16)
  //   e_dist  [2][ne] arclen(ed%c, tr(ed%sh(i))%c) (scalar_tr2ed's bary
  //           weights, pxt16; the dtred interpolation)
  //   t_edarea [3][nt] sphtriarea(tr%c, the end cells of triangle edge s)
  //           (scalar_edtr2trcc, geodesic areas; gass18)
  //   e_stq   [kMaxSt][ne] per TRSK stencil slot the connecting edge
  //           gethxedgeconnection(e, k) (smeshpack.f90:4174-4244) whose PV the
  //           gass Coriolis term takes, or -1 for the TRSK average (gass18)
  //   e_nr    [3][ne] ed%nr (pered, dtred)
  HVec<double> t_bary, e_dist, t_edarea, e_nr;
  HVec<int32_t> e_stq;
  // ... and their FP32 forms for the FP32 step (variant 0), each constant
  // factor folded in FP64 and rounded once:
  //   t_kite32 holds the depth weights of the triangle's vertices instead of
  //           the kite fractions: tr%c%b (pxt16) or, for gass18, half the
  //           edge areas of the two triangle edges at the vertex over A
  //   e_qw32  [2][ne] weights of q_e from the edge's triangles: d2, d1 over
  //           d1 + d2 (pxt16), a1, a2 over a1 + a2 (gass18, rhombus PV)
  //   e_stc32 (pxt16) the pered coefficients of the TRSK stencil slots: at
  //           each of the edge's cells c, -(1/4) ttgout (ed%c%p - v%p) . nr_e
  //           edhx%leng / hx%areag, so that sum_k c_k F_k (q_e + q_k) is the
  //           -(v . nr) of coriolis_ed's pered branch (the tangent-plane
  //           projections drop out: nr_e is normal to the edge midpoint and
  //           both cells, which also zeroes the edge's own term)
  //   e_dtc32 [6][ne] (dtred) per triangle i of the edge and its edge slot s,
  //           -w_i sign(tr%tg) l_s (tr%c x ed(s)%c) . nr_e / tr%areag, w_i =
  //           d2, d1 over d1 + d2: the PV flux is sum q_i c_is F_s
  HVec<float> e_qw32, e_dtc32;
  // c_C32 [36][nv] (pxt16, the cell-centred variants) the pered coefficients
  //           by cell: c_C32[6 i + j] couples the flux F_j (q_i + q_j) of
  //           the cell's slot-j edge into the PV flux of its slot-i edge,
  //           times that edge's ed%leng (the edge kernel divides the sum of
  //           its two cells' contributions by l_e)
  HVec<float> c_C32;
  // c_gout [6][nv] (gass18, the cell-centred variants) the outer edge of
  //           the cell's triangle in each slot (device index).  gass18's
  //           connecting edge of the cell's edge pair (i, j)
  //           (edge_connection) is that of triangle i for j = i + 1 (of
  //           triangle j for j = i - 1), the cell's edge i + 1 for j = i + 2
  //           (i - 1 for j = i - 2) and none for opposite edges; gass_cells
  //           is true when every cell is a pentagon or hexagon that follows
  //           this rule (checked against edge_connection pair by pair), and
  //           only then do the cell-centred variants run gass18
  HVec<int32_t> c_gout;
  bool gass_cells = false;
  // c_qw32 [6 slots][2][nv] (pxt16, the cell-centred variants)
  //           e_qw32 by cell slot: the weights of the slot's triangles j - 1
  //           and j in its edge's q_e
  HVec<float> c_qw32;
  // dtred in the cell-centred variants: t_dpa32 [3 slots][3][nt] the
  //           Perot weights a_ts = sign(tr%tg) l_s (tr%c x ed(s)%c) /
  //           tr%areag of the triangle's edges (P_t = sum_s uh_s a_ts);
  //           t_dopp [nt] the corner opposite edge slot s in bits 2s, 2s+1;
  //           e_nr32 [3][ne] ed%nr; e_dw32 [2][ne] d2, d1 over d1 + d2.  The
  //           PV flux is -sum_i w_i q_ti (P_ti . nr_e)
  HVec<float> t_dpa32, e_nr32, e_dw32;
  HVec<uint8_t> t_dopp;
};

// Builds the layout from a reference mesh; returns "" or an error message.
// scheme (IMODEL_SWM_TRSK10 ... IMODEL_SWM_DTRED) selects the extra geometry;
// fsphere = 2 sets f = fcte at every triangle instead of 2 Omega sin(lat).
std::string build_layout(const imodel_swm_mesh &m, const double *bt, Layout &L,
                         int scheme = IMODEL_SWM_TRSK10, int fsphere = 0, double fcte = 0.0);

// Inputs of the learned TRSK correction (imodel_gb300/learned.py), device
// order: per edge the 10 stencil edges as sign * (index + 1) (0 = padding),
// slot-major [10][ne], and the 14 geometry inputs as BF16 bit patterns,
// [ne][16] (two zero pads, 32 bytes per edge).
// Inputs of the learned correction, one 11,264-byte block per tile of 128
// edges (ntiles = ceil(ne / 128); padding rows: empty stencil slots, zero
// geometry, triangle and cell 0), so that a tile's inputs are one bulk copy:
//   int32 lst[10][128]  sign * (edge + 1) of the stencil slots, 0 = empty
//   bf16  geo[128][16]  geometry inputs (14 used)
//   int32 esh[2][128]   the edge's triangles
//   uint32 evs[128][2]  the edge's cell words
struct LearnedLayout {
  static constexpr int kTile = 128, kBlockBytes = 11264;
  static constexpr int kLst = 0, kGeo = 5120, kEsh = 9216, kEvs = 10240;
  int64_t ntiles = 0;
  HVec<uint8_t> blocks;  // [ntiles][kBlockBytes]
};
std::string build_learned_layout(const imodel_swm_mesh &m, const Layout &L, LearnedLayout &LL);

// The arrays of a trsk10 layout that depend on the TRSK weights and kite
// fractions (e_stw, e_stc32, c_R32, c_pk), for mesh m whose topology and
// node positions are those L was built from (so L's orderings hold): what
// build_layout would give for m, without building the rest again.
struct WeightArrays {
  HVec<double> e_stw;
  HVec<float> e_stc32, c_R32;
  HVec<int32_t> c_pk;
};
std::string build_weight_arrays(const imodel_swm_mesh &m, const Layout &L, WeightArrays &W);

// float -> BF16 bit pattern, round to nearest, ties to even
uint16_t bf16_bits(float v);

// Inputs of the learned TRSK weights (imodel_gb300/learned_weights.py): 24
// BF16 geometry features for every kite slot j < nnb of every cell,
// slot-major (all slot-0 kites, then slot 1, ...), and each row's cell and
// slot (0-based, reference numbering).
struct KiteInputs {
  HVec<uint16_t> x;    // [n][24]
  HVec<int32_t> cell;  // [n]
  HVec<int8_t> slot;   // [n]
};
std::string build_kite_inputs(const imodel_swm_mesh &m, KiteInputs &K);
// Kite fractions R' = R + 0.1 y (y the network outputs, projected to sum
// zero over each cell's slots) and the TRSK weights rebuilt from them
// (calc_trisk_weights, interpack.f90:4046-4095), in the mesh's layout:
// hxtr[nv][6], trskw[nv][6][6] with trskw(i, j) at [c][j][i].
void apply_kite_outputs(const imodel_swm_mesh &m, const KiteInputs &K, const float *y,
                        HVec<double> &hxtr, HVec<double> &trskw);

}  // namespace imodel
