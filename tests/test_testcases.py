"""Initial states of test cases 0, 1, 5 and 6 (imodel_gb300/testcases.py)
and the truncation error of the discrete tendency against the analytic
case-6 tendency, computed by the oracle (the GPU FP64 path equals the oracle
bit for bit, tests/test_gpu_testcases.py)."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import testcases as tc
from imodel_gb300.mesh import ERAD


def rel_l2(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b ** 2)))


def test_case0_and_case1_fields(grid_at):
    g = grid_at(5)
    h, u, bt = tc.initialize_fields(g, 0)
    assert np.all(u == 0) and np.all(bt == 0)
    assert abs(h.max() - 1.0) < 1e-2 and abs(h.min() + 1.0) < 1e-2
    h, u, bt = tc.initialize_fields(g, 1)
    lon, lat = tc.lonlat(g.v_p)
    r = ERAD * tc.arclen(g.v_p, tc.sph2cart(0.0, 0.0))
    assert np.all(h[r >= ERAD / 3.0] == 0.0)
    assert 990.0 < h.max() <= 1000.0
    # solid-body rotation: u = u0 cos(lat) e_lon . tg, at most u0 (with the
    # reference's pi, built from a float32 literal)
    assert np.abs(u).max() <= 2.0 * tc.PI * ERAD / (12 * 86400.0) + 1e-9


def test_case5_mountain(grid_at):
    g = grid_at(6)
    h, u, bt = tc.initialize_fields(g, 5)
    k = np.argmax(bt)
    lon, _ = tc.lonlat(g.v_p)
    assert abs(lon[k] + np.pi / 2) < 0.05 and abs(g.v_lat[k] - np.pi / 6) < 0.05
    assert 1800.0 < bt.max() <= 2000.0 and bt.min() == 0.0
    # the free surface h + b is the zonal-flow surface, unaffected by the cone
    s = np.sin(g.v_lat)
    h_ct = (ERAD * 7.292e-5 * 20.0 + 200.0) / 9.80616
    np.testing.assert_allclose(h + bt, 5960.0 - h_ct * s * s, rtol=0, atol=1e-9)


def test_case6_fields_match_analytic_wave(grid_at):
    g = grid_at(5)
    h, u, bt = tc.initialize_fields(g, 6)
    # wave pattern: h varies with 4 lon periods along a latitude circle
    lon, _ = tc.lonlat(g.v_p)
    band = np.abs(g.v_lat - np.radians(30.0)) < 0.03
    c = np.corrcoef(h[band], np.cos(4 * lon[band]))[0, 1]
    assert c > 0.99
    assert h.min() == 8000.0 and h.max() < 11000.0  # h0 at the poles


def test_case6_truncation_error_converges(grid_at):
    """masseq converges at first order or better in L2 on these grids; the
    TRSK momentum tendency converges slowly in L2 (its maximum error does not
    converge on grids without optimisation, a known property of TRSK on
    icosahedral grids)."""
    oracle.build()
    em, eu = [], []
    for level in (3, 4, 5, 6):
        g = grid_at(level)
        h, u, _ = tc.initialize_fields(g, 6)
        mex, uex = tc.tc6_exact_tendency(g)
        m, mo = oracle.Oracle(g, 6).tendency(h, u)
        em.append(rel_l2(m, mex, g.hx_areag))
        eu.append(rel_l2(mo, uex, g.ed_leng * g.edhx_leng))
    print("case 6 truncation error, levels 3-6: masseq", ["%.3e" % x for x in em],
          "momeq", ["%.3e" % x for x in eu])
    for a, b in zip(em, em[1:]):
        assert a / b > 1.8
    for a, b in zip(eu, eu[1:]):
        assert a / b > 1.2
    assert em[-1] < 0.1 and eu[-1] < 0.3


def test_unknown_case_is_refused(grid_at):
    with pytest.raises(ValueError):
        tc.initialize_fields(grid_at(2), 58)
    with pytest.raises(ValueError):
        tc.matsuno_parameters(2)


def test_matsuno_dispersion_relation():
    """Cases 56/57 (swm_matsuno.f90): the three frequencies solve the
    equatorial beta-plane cubic w^3 - (c^2 k^2 + beta c (2n+1)) w - beta c^2
    k = 0; the inertia-gravity wave takes the largest, the Rossby wave the
    smallest in magnitude, with the periods the reference's analysis uses
    (1.9 and 18.5 days)."""
    c = np.sqrt(tc.GRAV * tc.MATSUNO_H0)
    beta = 2.0 * tc.OMEGA / tc.ERAD
    k = tc.MATSUNO_K / tc.ERAD
    n = tc.MATSUNO_N
    A, B = c * c * k * k + beta * c * (2 * n + 1), beta * c * c * k
    w56 = tc.matsuno_parameters(56)[0]
    w57 = tc.matsuno_parameters(57)[0]
    for w in (w56, w57):     # the Rossby root is negative: w = -min |w_nk| is that root
        # Cardano's form loses a few digits to cancellation on the small root
        assert abs(w ** 3 - A * w - B) < 1e-5 * (A * abs(w) + B)
    assert w56 > 0 and w57 < 0
    assert abs(2 * np.pi / w56 / tc.DAY2SEC - 1.9) < 0.05
    assert abs(2 * np.pi / -w57 / tc.DAY2SEC - 18.5) < 0.05


def test_hermite_functions_are_orthonormal():
    x = np.linspace(-12.0, 12.0, 24001)
    dx = x[1] - x[0]
    hs = [tc.hermite(x, n) for n in range(4)]
    for i in range(4):
        for j in range(4):
            v = np.sum(hs[i] * hs[j] * np.exp(-x * x)) * dx
            assert abs(v - (1.0 if i == j else 0.0)) < 1e-6


@pytest.mark.parametrize("case,dt", [(56, 300.0), (57, 1800.0)])
def test_matsuno_wave_propagates(grid_at, case, dt):
    """A quarter period in the oracle at levels 4 and 5: h stays close to the
    travelling exact wave (persistence would be 141 % off) and the error
    falls with resolution."""
    w = tc.matsuno_parameters(case)[0]
    n = int(round(2 * np.pi / abs(w) / 4 / dt))
    err = []
    for level in (4, 5):
        g = grid_at(level)
        h0, u0, _ = tc.initialize_fields(g, case)
        h, _ = oracle.Oracle(g, case).run(h0, u0, dt, n)
        he, _ = tc.matsuno_fields(g, case, n * dt)
        a = g.hx_areag
        err.append(np.sqrt(np.sum(a * (h - he) ** 2) / np.sum(a * (he - tc.MATSUNO_H0) ** 2)))
    assert err[0] < 0.1 and err[1] < 0.7 * err[0]


def test_galewsky_jet(grid_at):
    """Cases 21-23: 10 km mean depth, the jet's maximum at 45 degrees, the
    height bump only in 21 and 23, and case 22 (no bump) in balance: its
    discrete momentum tendency is small beside the pressure gradient it
    balances."""
    g = grid_at(6)
    A = g.hx_areag
    h22, u22, _ = tc.initialize_fields(g, 22)
    h21, u21, _ = tc.initialize_fields(g, 21)
    h23, u23, _ = tc.initialize_fields(g, 23)
    assert abs(np.sum(A * h22) / np.sum(A) - 1.0e4) < 1.0
    assert 79.0 < np.abs(u22).max() <= 80.0 and 198.0 < np.abs(u23).max() <= 200.0
    assert np.array_equal(u21, u22)
    bump = h21 - h22
    k = np.argmax(bump)
    lon, _ = tc.lonlat(g.v_p)
    # 120 m cos(lat) exp(...): at most 120 cos(45 degrees) at the centre
    assert 80.0 < bump.max() <= 120.0 * np.cos(np.pi / 4) + 1e-9
    assert abs(lon[k]) < 0.1 and abs(g.v_lat[k] - np.pi / 4) < 0.1
    oracle.build()
    o = oracle.Oracle(g, 22)
    m, mo = o.tendency(h22, u22)
    grad = o.field("grad_ghbK")
    assert np.sqrt(np.mean(mo ** 2)) < 0.05 * np.sqrt(np.mean(grad ** 2))


def test_localised_steady_states_converge(grid_at):
    """Cases 40-42 are steady states of the continuous equations on an
    f-sphere: the discrete momentum tendency, relative to the height
    gradient it balances, falls with resolution."""
    for case in (40, 41, 42):
        res = []
        for L in (4, 5, 6):
            g = grid_at(L)
            h, u, bt = tc.initialize_fields(g, case)
            o = oracle.Oracle(g, bt=bt, **tc.case_options(case))
            _, mo = o.tendency(h, u)
            res.append(np.abs(mo).max() / np.abs(o.field("grad_ghbK")).max())
        assert res[0] > res[1] > res[2], (case, res)


def test_f_sphere_option_sets_constant_f(grid_at):
    """fsphere = 2 adds the constant fcte to the relative vorticity in place
    of 2 Omega sin(lat) (vort_tr, swm_operators.f90:592-601)."""
    g = grid_at(3)
    h, u, bt = tc.initialize_fields(g, 42)
    a = oracle.Oracle(g, 42, fsphere=2, fcte=1.4584e-4)
    b = oracle.Oracle(g, 42, fsphere=2, fcte=0.0)
    a.tendency(h, u)
    b.tendency(h, u)
    np.testing.assert_allclose(a.field("eta") - b.field("eta"), 1.4584e-4, rtol=1e-9, atol=0)
    np.testing.assert_allclose(b.field("eta"), b.field("zeta"), rtol=1e-13, atol=1e-20)


def test_southern_jet_and_its_bump(grid_at):
    g = grid_at(6)
    h52, u52, _ = tc.initialize_fields(g, 52)
    h53, u53, _ = tc.initialize_fields(g, 53)
    assert np.array_equal(u52, u53)
    # the jet lies between 45 and 5 degrees south and peaks at 80 m/s
    lat = np.degrees(g.ed_c_lat)
    assert np.all(np.abs(u52[(lat > -4.9) | (lat < -45.1)]) < 1e-12)
    assert 75.0 < np.abs(u52).max() <= 80.0
    # 53 adds the 120 m bump centred at (-120, -25) degrees
    d = h53 - h52
    k = np.argmax(d)
    lon, _ = tc.lonlat(g.v_p)
    assert 100.0 < d.max() <= 120.0
    assert abs(np.degrees(lon[k]) + 120.0) < 3.0 and abs(np.degrees(g.v_lat[k]) + 25.0) < 3.0


def test_hollingsworth_and_case51_layers(grid_at):
    g = grid_at(5)
    s = np.sin(g.v_lat)
    u0 = 2.0 * tc.PI * ERAD / (12 * 86400.0)
    for case in (32, 33):
        h, u, bt = tc.initialize_fields(g, case)
        assert np.all(h == tc.HOLLGW)
        # a divergence-free zonal flow: the mass tendency is truncation error
        # only, far below the scale h u0 / a of its terms
        o = oracle.Oracle(g, bt=bt, **tc.case_options(case))
        m, _ = o.tendency(h, u)
        assert np.abs(m).max() < 1e-2 * tc.HOLLGW * u0 / ERAD
    h32, _, b32 = tc.initialize_fields(g, 32)
    h33, _, b33 = tc.initialize_fields(g, 33)
    assert np.all(b33 >= b32)   # the f = 0 balance needs a smaller pole-equator drop
    h, u, bt = tc.tc51(g, hollgw=50.0)
    h_ct = (ERAD * 7.292e-5 * 20.0 + 200.0) / 9.80616
    np.testing.assert_allclose(h + bt, 50.0 + 5960.0 - h_ct * s * s, rtol=0, atol=1e-9)
    assert 49.0 - 20.0 < h.min() < 31.0


def test_unavailable_cases_are_named():
    with pytest.raises(ValueError, match="ENDGame"):
        tc.initialize_fields(None, 24)
    with pytest.raises(ValueError, match="ETOPO"):
        tc.initialize_fields(None, 60)
