"""The grid builder against an output of the reference itself.

The reference ships the figure of one run of its divergence test
(doc/divtest_f5_HC_error_icos_pol_nopt_5.pdf, made by gmt/plot.sh from the
run's field dump, doc/manual.tex:420-431): the error of the "HC" divergence
(velocities at the Voronoi-edge midpoints) of vector field 5 on the grid
icos_pol_nopt_5.  The test (simulpack.f90 divergence_test, :1006-1328)
evaluates the field at mesh%edhx(k)%c, projects it on mesh%edhx(k)%nr and
sums hx%nr(j) (v . nr) edhx%leng over each cell, divided by hx%areag
(diffoperpack.f90 div_cell_fullvec, :971-1073, pos 3); the exact divergence
of field 5 is zero, so the plotted error is minus that sum.  Field 5 is the
zonal flow u(lat) = cos(lat) with v = 0 (simulpack.f90 vecfield, :3379-3548,
whose "!*dsin(lat)" shows the run's u = cos(lat) sin(lat)).

The figure's colour bar is symmetric (grd2cpt -T=, gmt/plot.sh:514-524) with
labels at k/5 of the largest |error| for k = 1..5: 8.2e-05, 1.6e-04,
2.5e-04, 3.3e-04, 4.1e-04.  Rounded to two digits, those five labels hold
together only for a largest |error| in [4.0833e-4, 4.125e-4).  The same
divergence on this library's icos_pol_nopt_5 (nodes, Voronoi-edge midpoints,
normals, lengths, areas and signs from imodel_mesh_build) must fall in that
interval: a 1 % pin of the grid geometry against the reference's own run.
(With u = cos(lat), the field as the current source has it, the largest
error is 2.20e-4, outside the interval: the figure predates that edit.)
"""
import numpy as np
import pytest

from imodel_gb300.mesh import meshbuild


def hc_divergence(g, u_of_lat):
    """div_cell_fullvec (pos 3) of the zonal field u(lat) east, v = 0,
    evaluated at the Voronoi-edge midpoints (vecfield + proj_vec_sphere)."""
    p = g.edhx_c.reshape(-1, 3)
    pn = p / np.linalg.norm(p, axis=1)[:, None]
    lon = np.arctan2(pn[:, 1], pn[:, 0])
    lat = np.arcsin(np.clip(pn[:, 2], -1.0, 1.0))
    u = u_of_lat(lat)
    vec = np.stack([-np.sin(lon) * u, np.cos(lon) * u, np.zeros_like(lon)], axis=1)
    vec = vec - np.sum(vec * pn, axis=1)[:, None] * pn
    vn = np.sum(vec * g.edhx_nr.reshape(-1, 3), axis=1)
    ved = g.v_ed.reshape(-1, 6).astype(np.int64) - 1
    hxnr = g.hx_nr.reshape(-1, 6).astype(np.float64)
    div = np.zeros(g.nv)
    for j in range(6):
        m = j < g.nnb
        k = ved[m, j]
        div[m] += hxnr[m, j] * vn[k] * g.edhx_leng[k]
    return div / g.hx_areag


# the interval the figure's five colour-bar labels allow (see above)
LABELS = (8.2e-5, 1.6e-4, 2.5e-4, 3.3e-4, 4.1e-4)


def label_interval():
    lo, hi = 0.0, np.inf
    for k, lab in enumerate(LABELS, start=1):
        lo = max(lo, (lab - 0.05 * 10.0 ** np.floor(np.log10(lab))) * 5 / k)
        hi = min(hi, (lab + 0.05 * 10.0 ** np.floor(np.log10(lab))) * 5 / k)
    return lo, hi


def test_label_interval():
    lo, hi = label_interval()
    assert lo == pytest.approx(4.0833e-4, rel=1e-4) and hi == pytest.approx(4.125e-4, rel=1e-9)


def test_divergence_test_figure_icos_pol_nopt_5():
    g = meshbuild(5, "pol")
    assert g.nv == 10242
    err = -hc_divergence(g, lambda lat: np.cos(lat) * np.sin(lat))
    lo, hi = label_interval()
    m = float(np.max(np.abs(err)))
    print(f"largest |error| {m:.5e}, the figure allows [{lo:.5e}, {hi:.5e})")
    assert lo <= m < hi
    # the colour bar is symmetric because the error is: the largest
    # positive and negative errors have the same size
    assert float(err.max()) == pytest.approx(-float(err.min()), rel=1e-6)
