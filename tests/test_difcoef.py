"""The "align" and "diam" diffusion coefficient fields (alignment_coef,
diameter_coef, swm_operators.f90:977-1069; alignind, smeshpack.f90:
6398-6490) against a per-cell loop restatement of the Fortran, their
properties on the icosahedral meshes, and the oracle's diffusion with
coefficient fields."""
import math

import numpy as np
import pytest

import oracle
from imodel_gb300 import difcoef, fields, swm
from imodel_gb300.testcases import arclen


def _loop_fields(g, k_max):
    """Cell by cell, as the Fortran loops run (1-based slots shifted)."""
    cc = difcoef.circumcentres(g)
    diam = np.zeros(g.nv)
    ali = np.zeros(g.nv)
    for i in range(g.nv):
        n = int(g.nnb[i])
        tr = [int(g.v_tr[i, j]) - 1 for j in range(n)]
        d = 0.0
        for j in range(n):
            for k in range(n):
                d = max(d, float(arclen(cc[tr[j]], cc[tr[k]])))
        diam[i] = d
        if n == 6:
            tmp, meanl = 0.0, 0.0
            for j in range(1, 4):
                i1, i2, i3 = tr[j - 1], tr[j], tr[j + 2]
                i0 = tr[(j + 4 - 1) % 6]
                t1 = float(arclen(cc[i1], cc[i2]))
                t2 = float(arclen(cc[i3], cc[i0]))
                meanl = t1 + t2
                tmp = tmp + abs(t1 - t2)
                t1 = float(arclen(cc[i1], cc[i0]))
                t2 = float(arclen(cc[i2], cc[i3]))
                tmp = tmp + abs(t1 - t2)
            ali[i] = (tmp / 6) / (meanl / 6)
        else:
            ali[i] = 1.0
    sm = np.zeros(g.nv)
    for i in range(g.nv):
        s = ali[i]
        for j in range(int(g.nnb[i])):
            s = s + ali[int(g.v_nb[i, j]) - 1]
        sm[i] = s / (int(g.nnb[i]) + 1.0)
    p = math.log(10.0) / math.log(2.0)
    return (k_max * (sm / sm.max()),
            k_max * np.power(diam / diam.max(), p))


@pytest.mark.parametrize("level", [1, 2])
def test_fields_equal_the_loop_restatement(grid_at, level):
    g = grid_at(level)
    a_ref, d_ref = _loop_fields(g, 3.0e5)
    np.testing.assert_allclose(difcoef.alignment_coef(g, 3.0e5), a_ref, rtol=1e-14, atol=0)
    np.testing.assert_allclose(difcoef.diameter_coef(g, 3.0e5), d_ref, rtol=1e-14, atol=0)


def test_field_properties(grid_at):
    g = grid_at(4)
    k = 1.0e5
    d = difcoef.diameter_coef(g, k)
    assert d.max() == k and d.min() > 0
    diam = difcoef.diameter(g)
    p = math.log(10.0) / math.log(2.0)
    np.testing.assert_allclose(d.min() / d.max(), (diam.min() / diam.max()) ** p, rtol=1e-12)
    a = difcoef.alignment_coef(g, k)
    assert a.max() == k and a.min() > 0
    pent = g.nnb == 5
    assert pent.sum() == 12
    # the pentagons' index is 1, far above any hexagon's: after smoothing
    # they carry the largest coefficients, equal by symmetry
    assert np.all(a[pent] > (1 - 1e-9) * k) and np.all(a[~pent] < a[pent].min())


def test_constant_field_is_the_constant_path(grid_at):
    g = grid_at(3)
    h, u = fields.balanced_state(g, lmax=8, seed=9)
    for k2, k4 in ((1.0e5, 0.0), (0.0, 1.0e14), (1.0e5, 1.0e13)):
        _, ma = oracle.Oracle(g, 2, k2=k2, k4=k4).tendency(h, u)
        _, mb = oracle.Oracle(g, 2, k2_hx=np.full(g.nv, k2) if k2 else None,
                              k4_hx=np.full(g.nv, k4) if k4 else None).tendency(h, u)
        assert np.array_equal(ma, mb)


def test_field_diffusion_takes_energy_out(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=10)
    w = 0.5 * g.ed_leng * g.edhx_leng
    _, m0 = oracle.Oracle(g, 2).tendency(h, u)
    for f in (difcoef.diameter_coef, difcoef.alignment_coef):
        _, m2 = oracle.Oracle(g, 2, k2_hx=f(g, 1.0e5)).tendency(h, u)
        _, m4 = oracle.Oracle(g, 2, k4_hx=f(g, 1.0e14)).tendency(h, u)
        assert np.sum(w * u * (m2 - m0)) < 0 and np.sum(w * u * (m4 - m0)) < 0


def test_bad_fields_refused(grid_at):
    g = grid_at(2)
    f = np.full(g.nv, 1.0e5)
    f[3] = -1.0
    with pytest.raises(ValueError):
        oracle.Oracle(g, 2, k2_hx=f)
    f[3] = np.nan
    with pytest.raises(ValueError):
        oracle.Oracle(g, 2, k4_hx=f)
