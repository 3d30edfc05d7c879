/*
 * imodel_mesh.h -- icosahedral Voronoi/Delaunay grid builder (host C++,
 * with a GPU back end for the geometry).
 *
 * Builds the grid_structure fields that the shallow-water step consumes, for
 * the non-optimised hierarchical icosahedral grids of iModel:
 *
 *   icosanodes0   src/smeshpack.f90:1197-1296  (12 base nodes, eqs / pol)
 *   meshrefin     src/smeshpack.f90:1587-1675  (edge midpoints, normalised)
 *   meshstruct    src/smeshpack.f90:370-1195   (edges, triangles, Voronoi
 *                                                cells, signs, areas)
 *   trhx_intersec_areas / hxtr_intersec_areas
 *                 src/smeshpack.f90:5080-5154, :4991-5078
 *   calc_trisk_weights  src/interpack.f90:3978-4098
 *
 * The reference re-triangulates every level with STRIPACK (trmesh,
 * stripackm.f90:6843).  For midpoint-refined icosahedral nodes that
 * triangulation is the 4-way subdivision of the previous one; the builder
 * uses the subdivision and verifies the Delaunay empty-circumcircle property
 * on every edge (imodel_mesh_delaunay_violations).  Values per entity are the
 * reference's; the numbering of nodes appended at a level and the starting
 * neighbour of each ccw list may differ, because they follow STRIPACK's
 * internal list order in the reference.
 *
 * All index arrays are 1-based and laid out as documented in imodel_swm.h.
 */
#ifndef IMODEL_MESH_H
#define IMODEL_MESH_H

#include <stdint.h>
#include "imodel_swm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque grid owned by the library.  level: icosahedral refinement level
 * (nv = 10*4^level + 2).  pos: 0 = "eqs" (equator symmetric), 1 = "pol"
 * (nodes on the poles).  nthreads: host threads for the geometry loops
 * (0 = all).  Returns 0 or an IMODEL_SWM_E* code. */
int imodel_mesh_build(int32_t level, int32_t pos, int32_t nthreads,
                      void **grid);

/* The same grid built on CUDA device `device`: the subdivision (meshrefin,
 * smeshpack.f90:1587-1675), the neighbour rings and meshstruct's numbering
 * of edges and triangles (:706-862) by kernels that hand out
 * imodel_mesh_build's numbers, then one GPU kernel per meshstruct step forms
 * every length, area, angle, sign, kite fraction and TRSK weight, and the
 * Delaunay check (smeshpack.f90:706-1151, :4991-5154; interpack.f90:
 * 3978-4098).  Node positions, index and sign arrays equal
 * imodel_mesh_build's bit for bit; the GPU's atan, tan, atan2 and
 * asin may differ from the host C library's in the last bit, so lengths,
 * areas, angles and weights agree with imodel_mesh_build's to a few units in
 * the last place.  The result is an ordinary grid handle (view, extra_view,
 * delaunay_violations, free).  Returns 0, IMODEL_SWM_EINVAL,
 * IMODEL_SWM_ENOMEM or IMODEL_SWM_ECUDA (message from
 * imodel_mesh_gpu_last_error, per calling thread). */
int imodel_mesh_build_gpu(int32_t level, int32_t pos, int32_t device,
                          void **grid);
const char *imodel_mesh_gpu_last_error(void);

/* Fills *view with pointers into the grid's arrays (valid until free). */
int imodel_mesh_view(void *grid, imodel_swm_mesh *view);

/* Extra per-entity geometry not needed by the time step (for initial states
 * and diagnostics): cell lon, edge midpoint lon, triangle circumcentres
 * [nt][3], Voronoi-edge midpoints [ne][3], edhx%nr/tg [ne][3]. */
typedef struct imodel_mesh_extra {
  const double *v_lon;
  const double *ed_c_lon;
  const double *tr_c;
  const double *edhx_c;
  const double *edhx_nr;
  const double *edhx_tg;
  const int32_t *hx_nr;  /* [nv][6] hx%nr (+-1) */
  const int32_t *tr_nr;  /* [nt][3] tr%nr (+-1) */
} imodel_mesh_extra;
int imodel_mesh_extra_view(void *grid, imodel_mesh_extra *view);

/* Number of Delaunay violations found (edges whose opposite vertex lies
 * strictly inside the neighbour triangle's circumcircle) and the smallest
 * in-circle margin seen (positive = Delaunay with that margin). */
int imodel_mesh_delaunay_violations(void *grid, int64_t *count,
                                    double *min_margin);

void imodel_mesh_free(void *grid);

#ifdef __cplusplus
}
#endif
#endif /* IMODEL_MESH_H */
