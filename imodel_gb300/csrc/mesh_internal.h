// Internal to the grid builder: the grid the library hands out and the
// topology both geometry back ends (host loops in mesh.cpp, GPU kernels in
// mesh_gpu.cu) start from.  Not part of the C ABI.
#pragma once

#include <cstdint>
#include <vector>

namespace imodel {
namespace mesh {

// The grid_structure arrays of one grid, 1-based index arrays padded with 0
// (the layouts of include/imodel_swm.h and include/imodel_mesh.h).
struct Grid {
  int nv = 0, ne = 0, nt = 0;
  std::vector<int32_t> nnb, v_nb, v_ed, v_tr, ttgout, tnrccw, hx_nr;
  std::vector<int32_t> ed_v, ed_sh, tr_v, tr_ed, tr_tg, tr_nr;
  std::vector<double> hx_areag, hxtr, trskw, v_p, v_lat, v_lon;
  std::vector<double> ed_leng, edhx_leng, ed_c, ed_c_lat, ed_c_lon, ed_tg, ed_nr;
  std::vector<double> edhx_c, edhx_nr, edhx_tg;
  std::vector<double> tr_areag, tr_trhx, tr_c, tr_c_lat;
  int64_t delaunay_bad = 0;
  double delaunay_margin = 0.0;
};

// The combinatorial structure of a grid, 0-based (meshstruct's index
// arrays, smeshpack.f90:706-862): node positions and, per node, its ccw
// neighbours, edges and triangles (6 slots, -1 padded); per edge its two
// nodes (lower index first) and the two triangles sharing it (lower index
// first); per triangle its three nodes and its edges (edge l joins nodes l
// and l + 1 mod 3).
struct Topo {
  int nv = 0, ne = 0, nt = 0;
  std::vector<double> p;  // [nv][3]
  std::vector<int> nnb, ring, ved, vtr;  // [nv], [nv][6] x3
  std::vector<int> edv, edsh;  // [ne][2]
  std::vector<int> trv, tred;  // [nt][3]
};

// Nodes and topology of icos level `level` (pos 0 = "eqs", 1 = "pol");
// host threads (OpenMP).  Returns an IMODEL_SWM_* status.
int topology(int level, int pos, Topo &t);

// The 1-based index arrays of g from t (host threads).
void export_topology(const Topo &t, Grid &g);

// Geometry by the GPU kernels of mesh_gpu.cu on CUDA device `device`;
// `why` receives a message on a CUDA error.  Returns an IMODEL_SWM_* status.
int geometry_gpu(const Topo &t, Grid &g, int device, const char **why);

}  // namespace mesh
}  // namespace imodel
