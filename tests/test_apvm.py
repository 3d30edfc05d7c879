"""The anticipated potential vorticity method in the oracle (pv_stab =
"apvm", swm_operators.f90:1465-1543): off at pvspar 0, the PV gradient it
reads against the exact one of case 2, the Coriolis term still neutral for
the energy, and potential enstrophy taken out of the Galewsky jet."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import fields, swm
from imodel_gb300 import testcases as tc


def test_zero_parameter_is_the_plain_tendency(grid_at):
    g = grid_at(3)
    h, u = fields.balanced_state(g, lmax=8, seed=2)
    ma, ua = oracle.Oracle(g, 2).tendency(h, u)
    mb, ub = oracle.Oracle(g, 2, pvspar=0.0, dt=600.0).tendency(h, u)
    mc, uc = oracle.Oracle(g, 2, pvspar=0.5, dt=600.0).tendency(h, u)
    assert np.array_equal(ma, mb) and np.array_equal(ua, ub)
    assert np.array_equal(ma, mc) and not np.array_equal(ua, uc)


def test_bad_parameters_refused(grid_at):
    g = grid_at(2)
    for pv, dt in ((-1.0, 600.0), (0.5, 0.0), (0.5, -600.0), (float("nan"), 600.0)):
        with pytest.raises(ValueError):
            oracle.Oracle(g, 2, pvspar=pv, dt=dt)


def test_pv_gradient_of_solid_body_rotation(grid_at):
    """grad_tr2ed(q_tr) (swm_operators.f90:1427-1463) against grad q . ed%nr
    for case 2's q(lat) = 2 (u0/a + Omega) sin(lat) / h(lat): unbiased
    (median ratio 1), with a pointwise error near +-20 % that does not
    shrink -- the same first-order grid-scale error of a triangle field,
    differenced across one dual edge, as in the vector Laplacian.  The exact
    correction is zero there (grad q is meridional, v zonal); the discrete
    one stays about 3 % of 4 |grad q| |v|."""
    from imodel_gb300.mesh import ERAD
    u0, h0 = swm.tc2_constants()[:2]
    for level in (4, 5):
        g = grid_at(level)
        h, u = swm.initialize_fields_tc2(g)
        a = oracle.Oracle(g, 2)
        b = oracle.Oracle(g, 2, pvspar=1.0, dt=1.0)
        a.tendency(h, u)
        b.tendency(h, u)
        qg = b.field("q_grad_ed")
        om, grav = 7.292e-5, 9.80616

        def q(p):
            return 2.0 * (u0 / ERAD + om) * np.sin(p) / (
                h0 - (ERAD * om * u0 + 0.5 * u0 ** 2) * np.sin(p) ** 2 / grav)
        phi = g.ed_c_lat
        dq = (q(phi + 1e-6) - q(phi - 1e-6)) / 2e-6 / ERAD
        ex = swm.dot3(swm.convert_vec_sph2cart(0.0 * phi, dq, g.ed_c), g.ed_nr)
        big = np.abs(ex) > 0.3 * np.abs(ex).max()
        r = qg[big] / ex[big]
        assert abs(np.median(r) - 1.0) < 3e-3
        assert 0.7 < np.percentile(r, 5) and np.percentile(r, 95) < 1.35
        corr = a.field("q_ed") - b.field("q_ed")       # pvspar dt = 1
        assert np.abs(corr).max() < 0.05 * 4.0 * np.abs(dq).max() * u0


def test_coriolis_term_stays_energy_neutral(grid_at):
    """TRSK's PV flux does no work for any edge PV (the weights are
    antisymmetric and q enters as (q_e + q_k)/2), so the anticipated PV
    keeps sum_e l d uh_e (q u h)perp_e at rounding level."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=3)
    w = g.ed_leng * g.edhx_leng
    o = oracle.Oracle(g, 2, pvspar=1.0, dt=600.0)
    o.tendency(h, u)
    p = w * o.field("uh") * o.field("uhq_perp")
    assert abs(p.sum()) < 1e-13 * np.abs(p).sum()


def test_enstrophy_taken_out_of_the_galewsky_jet(grid_at):
    """Two days of case 21 at level 4 (dt 300 s): the potential enstrophy
    that plain TRSK gains on the unresolved jet shrinks as pvspar grows,
    while the total energy stays conserved."""
    g = grid_at(4)
    h, u, bt = tc.initialize_fields(g, 21)
    ens, eng = [], []
    for pv in (0.0, 0.5, 1.0):
        o = oracle.Oracle(g, 21, bt=bt, pvspar=pv, dt=300.0)
        o.tendency(h, u)
        d0 = o.diagnostics(h, u)
        hh, uu = o.run(h, u, 300.0, 576)
        o.tendency(hh, uu)
        d1 = o.diagnostics(hh, uu)
        ens.append(d1["pot_enstrophy"] / d0["pot_enstrophy"] - 1.0)
        eng.append(abs(d1["tenergy"] / d0["tenergy"] - 1.0))
    assert ens[0] > ens[1] > ens[2]
    assert max(eng) < 1e-7
