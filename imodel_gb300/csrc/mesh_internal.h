// Internal to the grid builder: the grid the library hands out and the
// topology both geometry back ends (host loops in mesh.cpp, GPU kernels in
// mesh_gpu.cu) start from.  Not part of the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace imodel {
namespace mesh {

// An allocator whose resize() leaves new elements uninitialised: every
// array of a grid is written in full by the parallel loops (or the GPU copy)
// that follow, so zero-filling it first on one thread is wasted time (about
// 0.5 s for the 12 GB of a level-10 grid) and would put every page on the
// first-touching thread's memory node.  assign(n, v) still fills.
template <class T>
struct NoInit : std::allocator<T> {
  using std::allocator<T>::allocator;
  template <class U>
  struct rebind {
    using other = NoInit<U>;
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
using Array = std::vector<T, NoInit<T>>;

// The grid_structure arrays of one grid, 1-based index arrays padded with 0
// (the layouts of include/imodel_swm.h and include/imodel_mesh.h).
struct Grid {
  int nv = 0, ne = 0, nt = 0;
  Array<int32_t> nnb, v_nb, v_ed, v_tr, ttgout, tnrccw, hx_nr;
  Array<int32_t> ed_v, ed_sh, tr_v, tr_ed, tr_tg, tr_nr;
  Array<double> hx_areag, hxtr, trskw, v_p, v_lat, v_lon;
  Array<double> ed_leng, edhx_leng, ed_c, ed_c_lat, ed_c_lon, ed_tg, ed_nr;
  Array<double> edhx_c, edhx_nr, edhx_tg;
  Array<double> tr_areag, tr_trhx, tr_c, tr_c_lat;
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

// The 12 nodes ([12][3]) and 20 counter-clockwise faces ([20][3], 0-based)
// of the level-0 icosahedron.  Returns an IMODEL_SWM_* status.
int level0(int pos, std::vector<double> &p, std::vector<int> &tri);

// The 1-based index arrays of g from t (host threads).
void export_topology(const Topo &t, Grid &g);

// Writes zeros over [p, p + bytes) on host threads, so that a buffer about
// to be filled by one copy has its pages mapped in parallel.
void touch(void *p, size_t bytes);

// Geometry by the GPU kernels of mesh_gpu.cu on CUDA device `device`;
// `why` receives a message on a CUDA error.  Returns an IMODEL_SWM_* status.
int geometry_gpu(const Topo &t, Grid &g, int device, const char **why);

// The whole grid on CUDA device `device`: the topology by kernels that give
// topology()'s numbers (and bit-identical node positions), then the
// geometry of geometry_gpu.  Returns an IMODEL_SWM_* status.
int build_gpu(int level, int pos, int device, Grid &g, const char **why);

}  // namespace mesh
}  // namespace imodel
