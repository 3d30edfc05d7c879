"""Per-cell diffusion coefficient fields of the "align" and "diam" branches of
swm_tests (swm.f90:169-205): alignment_coef and diameter_coef
(swm_operators.f90:977-1069) with the alignment index alignind
(smeshpack.f90:6398-6490).  They are set-up work on the host; the step takes
the fields through SWM.set_diffusion_fields / imodel_swm_set_diffusion_fields.

The triangles' circumcentres (tr%c%p) are the unit normals of their vertex
planes, on the vertices' side, the same points the library's layout uses."""
import numpy as np

from .mesh import Grid
from .testcases import arclen


def circumcentres(grid: Grid) -> np.ndarray:
    """[nt, 3] unit circumcentre directions of the triangles."""
    tv = grid.tr_v.astype(np.int64) - 1
    p0, p1, p2 = (grid.v_p[tv[:, k]] for k in range(3))
    a, b = p1 - p0, p2 - p0
    x = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                  a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                  a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)
    s = p0 + p1 + p2
    side = x[:, 0] * s[:, 0] + x[:, 1] * s[:, 1] + x[:, 2] * s[:, 2]
    nrm = np.sqrt(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1] + x[:, 2] * x[:, 2])
    return np.where((side < 0)[:, None], -x, x) / nrm[:, None]


def _cell_tri_points(grid: Grid, cc: np.ndarray):
    """[nv, 6, 3] circumcentres of each cell's triangles in v%tr order (the
    sixth slot of a pentagon repeats its first, never read by the callers)."""
    vt = grid.v_tr.astype(np.int64) - 1
    vt = np.where(vt < 0, vt[:, :1], vt)
    return cc[vt]


def diameter(grid: Grid) -> np.ndarray:
    """Cell diameters: the largest arc between two of the cell's triangle
    circumcentres (diameter_coef, swm_operators.f90:1048-1059)."""
    pts = _cell_tri_points(grid, circumcentres(grid))
    n = grid.nnb.astype(np.int64)
    d = np.zeros(grid.nv)
    for j in range(6):
        for k in range(6):
            ok = (j < n) & (k < n)
            a = arclen(pts[:, j], pts[:, k])
            d = np.where(ok, np.maximum(d, a), d)
    return d


def diameter_coef(grid: Grid, k_max: float) -> np.ndarray:
    """K_max (diam / max diam)^p, p = log 10 / log 2 (Zarzycki et al. 2014;
    swm_operators.f90:1026-1069)."""
    d = diameter(grid)
    d = d / d.max()
    p = np.log(10.0) / np.log(2.0)
    return k_max * np.power(d, p)


def alignind(grid: Grid) -> np.ndarray:
    """Alignment index of each cell (smeshpack.f90:6398-6490): for hexagons the
    mean mismatch of opposite Voronoi edge lengths and of the distances
    between them, over a sixth of the last pair's summed lengths (the
    reference overwrites that sum on each of the three passes); 1 for cells
    that are neither hexagons nor squares.  Icosahedral meshes have no
    squares."""
    pts = _cell_tri_points(grid, circumcentres(grid))
    tmp = np.zeros(grid.nv)
    meanl = np.zeros(grid.nv)
    for j in range(3):            # j = 1..3 in the reference
        i1, i2, i3, i0 = pts[:, j], pts[:, j + 1], pts[:, j + 3], pts[:, (j + 4) % 6]
        t1, t2 = arclen(i1, i2), arclen(i3, i0)
        meanl = t1 + t2
        tmp = tmp + np.abs(t1 - t2)
        t1, t2 = arclen(i1, i0), arclen(i2, i3)
        tmp = tmp + np.abs(t1 - t2)
    tmp = tmp / 6
    meanl = meanl / 6
    hexa = grid.nnb == 6
    with np.errstate(divide="ignore", invalid="ignore"):
        out = tmp / meanl
    if np.any(grid.nnb == 4):
        raise ValueError("alignind: square cells are not handled here")
    return np.where(hexa, out, 1.0)


def alignment_coef(grid: Grid, k_max: float) -> np.ndarray:
    """K_max times the alignment index averaged over the cell and its
    neighbours, over its maximum (swm_operators.f90:977-1024)."""
    a = alignind(grid)
    n = grid.nnb.astype(np.int64)
    nb = grid.v_nb.astype(np.int64) - 1
    s = a.copy()
    for j in range(6):
        s = np.where(j < n, s + a[np.where(nb[:, j] >= 0, nb[:, j], 0)], s)
    s = s / (n + 1.0)
    s = s / s.max()
    return k_max * s


FUNCTIONS = {"align": alignment_coef, "diam": diameter_coef}
