"""The learned correction inside the FP32 step: exact reduction to plain
TRSK with a zero network, the correction term against the host-side inputs,
and the energy-drift fallback."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import fields, learned, swm
from imodel_gb300.swm import SWM
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def test_zero_network_equals_plain_step(grid_at):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=24, seed=2)
    zero = np.zeros(mo.NPARAM, dtype=np.float32)
    a = SWM(g, "fp32", learned_params=zero)
    b = SWM(g, "fp32")
    b.set_tuning(variant=1)
    ha, ua = a.ode_rk4(h, u, 450.0, 10)
    hb, ub = b.ode_rk4(h, u, 450.0, 10)
    assert np.array_equal(ha, hb) and np.array_equal(ua, ub)
    assert a.diagnostics()["learned_active"] == 1


def test_correction_term_matches_host_inputs(grid_at):
    """momeq(learned) - momeq(plain) = q_e h_e sigma_e y_e with y from the
    network applied to the host-built inputs of the same velocity field."""
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=24, seed=4)
    p = mo.init_params(7)
    p[-1] = 0.05  # b3
    m1, mo1 = SWM(g, "fp32", learned_params=p).tendency(h, u)
    m0, mo0 = SWM(g, "fp32").tendency(h, u)
    assert np.array_equal(m1, m0)
    diff = mo1 - mo0
    o = oracle.Oracle(g, 2)
    o.tendency(h, u)
    x, sigma = learned.features(g, u)
    net = learned.Mlp(params=p)
    y = net.forward(learned.to_bf16_bits(x)).astype(np.float64)
    expect = o.field("q_ed") * o.field("h_ed") * sigma * np.clip(y, -learned.CORR_MAX,
                                                                    learned.CORR_MAX)
    err = np.max(np.abs(diff - expect)) / np.max(np.abs(expect))
    print(f"learned correction: max rel difference {err:.2e}")
    assert err < 2e-2


def test_energy_drift_guard_switches_off(grid_at):
    """A network far from the TRSK error destroys energy neutrality; once the
    drift exceeds the bound the plain scheme takes over.  (The error proxy
    would switch this network off at once: it moves the PV flux by far more
    than its bound.  A huge error_bound leaves the energy check alone.)"""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=16, seed=1)
    p = mo.init_params(8) * 50.0
    p[-1] = 30.0
    wild = SWM(g, "fp32", learned_params=p)
    wild.set_state(h, u)
    assert wild.diagnostics()["learned_active"] == 0
    assert wild.learned_error_proxy() > 0.25
    wild.close()
    m = SWM(g, "fp32", learned_params=p, drift_bound=1e-6, error_bound=1e30)
    m.set_state(h, u)
    assert m.diagnostics()["learned_active"] == 1
    for _ in range(20):
        m.advance(900.0, 5)
        if not m.diagnostics()["learned_active"]:
            break
    assert m.diagnostics()["learned_active"] == 0
    # a new run switches it on again
    m.set_state(h, u)
    assert m.diagnostics()["learned_active"] == 1


def test_guard_rolls_back_the_interval(grid_at):
    """An interval that breaks the bound is stepped again with the plain
    scheme: the result equals a plain run of the same steps bit for bit."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=16, seed=3)
    p = mo.init_params(9) * 50.0
    p[-1] = 30.0
    a = SWM(g, "fp32", learned_params=p, drift_bound=1e-12)
    b = SWM(g, "fp32")
    b.set_tuning(variant=1)
    ha, ua = a.ode_rk4(h, u, 900.0, 40)
    hb, ub = b.ode_rk4(h, u, 900.0, 40)
    assert a.diagnostics()["learned_active"] == 0
    assert np.array_equal(ha, hb) and np.array_equal(ua, ub)


def test_gather_group_splits_give_identical_steps(grid_at):
    """The network kernel's split of warps between gathering and the
    epilogue (2 to 4 gather groups) changes the schedule, not the
    arithmetic: the steps agree bit for bit."""
    from imodel_gb300 import learned as lrn
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=24, seed=9)
    p = lrn.trained_params()
    assert p is not None
    out = []
    for ng in (2, 3, 4):
        m = SWM(g, "fp32", learned_params=p)
        m.set_tuning(variant=2, mlp_gather=ng)
        out.append(m.ode_rk4(h, u, 450.0, 4))
    for hh, uu in out[1:]:
        assert np.array_equal(hh, out[0][0]) and np.array_equal(uu, out[0][1])
