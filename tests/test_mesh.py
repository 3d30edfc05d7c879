"""Grid builder: counts, known answers on the icosahedron, geometric and
TRSK-weight identities (smeshpack.f90 meshstruct, interpack.f90
calc_trisk_weights)."""
import math

import numpy as np
import pytest

import oracle
from imodel_gb300.mesh import nodes_at_level

FOURPI = 4.0 * math.pi


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5])
def test_counts_and_valence(grid_at, level):
    g = grid_at(level)
    nv = nodes_at_level(level)
    assert (g.nv, g.ne, g.nt) == (nv, 3 * nv - 6, 2 * nv - 4)
    assert np.sum(g.nnb == 5) == 12
    assert np.sum(g.nnb == 6) == nv - 12
    # every edge appears in exactly two cell lists and two triangles
    counts = np.bincount(g.v_ed[g.v_ed > 0] - 1, minlength=g.ne)
    assert np.all(counts == 2)
    assert np.all(g.ed_sh > 0) and np.all(g.ed_sh[:, 0] < g.ed_sh[:, 1])
    assert np.all(g.ed_v[:, 0] < g.ed_v[:, 1])


def test_icosahedron_known_answers(grid_at):
    """Level 0: 12 regular pentagons of area 4pi/12, 30 edges of arc
    acos(1/sqrt(5)), 20 triangles of area 4pi/20."""
    g = grid_at(0)
    np.testing.assert_allclose(g.ed_leng, math.acos(1 / math.sqrt(5)), rtol=1e-14)
    np.testing.assert_allclose(g.hx_areag, FOURPI / 12, rtol=1e-13)
    np.testing.assert_allclose(g.tr_areag, FOURPI / 20, rtol=1e-13)
    np.testing.assert_allclose(g.edhx_leng, g.edhx_leng[0], rtol=1e-13)
    # kites of a regular pentagon are equal: R = 1/5, w(i, j) = (j-i)/5 - 1/2
    np.testing.assert_allclose(g.hx_hxtr_area[:, :5], 0.2, rtol=1e-13)
    np.testing.assert_allclose(g.hx_trskw[0, 2, 0], 2 / 5 - 0.5, atol=1e-14)


@pytest.mark.parametrize("level", [1, 3, 5])
def test_area_identities(grid_at, level):
    g = grid_at(level)
    assert abs(g.hx_areag.sum() - FOURPI) < 1e-12
    assert abs(g.tr_areag.sum() - FOURPI) < 1e-12
    # L'Huilier loses relative precision on small triangles (~4^level * 1e-15)
    np.testing.assert_allclose(g.tr_trhx_area.sum(axis=1), g.tr_areag, rtol=1e-9)
    rs = np.array([g.hx_hxtr_area[i, :g.nnb[i]].sum() for i in range(g.nv)])
    np.testing.assert_allclose(rs, 1.0, rtol=1e-9)


@pytest.mark.parametrize("level", [2, 4])
def test_trsk_weights(grid_at, level):
    """w(i,j) = -w(j,i) (sum of kite fractions is 1) and the oracle's own
    restatement of calc_trisk_weights reproduces the builder's weights."""
    g = grid_at(level)
    w = g.hx_trskw  # [c, j, i]
    # exact up to (sum R - 1), the kite-area round-off
    np.testing.assert_allclose(w + np.transpose(w, (0, 2, 1)), 0.0, atol=1e-11)
    w2 = oracle.trsk_weights(g)
    assert np.array_equal(w, w2)


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5, 6])
def test_delaunay(grid_at, level):
    g = grid_at(level)
    assert g.delaunay_violations == 0
    assert g.delaunay_margin > 0


def test_hierarchical_numbering(grid_at):
    """Cell i of level L sits at the same point as cell i of level L+1."""
    for L in range(0, 4):
        a, b = grid_at(L), grid_at(L + 1)
        assert np.array_equal(a.v_p, b.v_p[:a.nv])


@pytest.mark.parametrize("level", [2, 4])
def test_flux_signs(grid_at, level):
    """The outward sign of an edge seen from its two cells is opposite, the
    discrete divergence theorem that makes mass conservation exact."""
    g = grid_at(level)
    sign = {}
    for i in range(g.nv):
        for j in range(g.nnb[i]):
            e = g.v_ed[i, j] - 1
            sign.setdefault(e, []).append(g.hx_ttgout[i, j])
    s = np.array([sum(v) for v in sign.values()])
    assert np.all(s == 0)


def test_pol_positions(grid_at):
    g = grid_at(2, "pol")
    assert np.allclose(g.v_p[0], [0, 0, 1])
    assert g.delaunay_violations == 0
    assert abs(g.hx_areag.sum() - FOURPI) < 1e-12


def _hashes():
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "mesh_hashes.json")
    with open(path) as f:
        return json.load(f)


@pytest.mark.parametrize("pos", ["eqs", "pol"])
@pytest.mark.parametrize("nthreads", [1, 0])
def test_builder_reproduces_the_pinned_grids(pos, nthreads):
    """Every array of the grids at levels 0-6 hashes to the fixture made
    with one thread (tests/golden/make_mesh_hashes.py): the numbering steps
    done as count + prefix sum + fill on many threads give the numbers of
    the serial sweep, and the geometry is bit for bit the same."""
    import importlib.util
    import os
    from imodel_gb300.mesh import meshbuild
    spec = importlib.util.spec_from_file_location(
        "make_mesh_hashes", os.path.join(os.path.dirname(__file__), "golden",
                                         "make_mesh_hashes.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    table = _hashes()
    for level in range(0, 7):
        got = mk.grid_hashes(meshbuild(level, pos, nthreads=nthreads))
        want = table[f"{pos}{level}"]
        diff = sorted(k for k in want if want[k] != got.get(k))
        assert not diff, (pos, level, diff)


def test_grid_arrays_outlive_the_grid():
    """The Grid's arrays view the library's grid without copying it; the
    grid is freed only when the last of them is gone."""
    import gc
    from imodel_gb300.mesh import meshbuild
    g = meshbuild(3)
    area, trskw = g.hx_areag, g.hx_trskw
    del g
    gc.collect()
    assert abs(float(area.sum()) - FOURPI) < 1e-12
    assert trskw.shape == (642, 6, 6) and np.all(np.isfinite(trskw))
    assert area.flags.writeable
