"""The learned TRSK weights on the GPU (imodel_swm_opts.learned = 2).

* the library computes the same corrected kite fractions and weights as the
  host pipeline (features, the tensor-core network, the rebuild);
* with those weights the FP64 step equals the oracle bit for bit, and the
  FP32 step (every stencil variant) stays within FP32 round-off of it;
* what the trained network gains: Williamson case 2 is a steady state, so
  the error of a run against its initial state is the scheme's own error;
  at levels the network was not trained on, the learned weights lower it;
* the guard's fallback rolls back to plain TRSK bit for bit, and the step
  costs the plain step's launches.
"""
import ctypes

import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, fields, learned, learned_weights as lw, swm
from imodel_gb300.swm import SWM, SWMError

pytestmark = pytest.mark.gpu


def _params():
    p = lw.trained_params()
    return p if p is not None else learned.init_params(7)


def rel(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b * b)))


def test_library_weights_match_the_host_pipeline(grid_at):
    g = grid_at(5)
    p = _params()
    m = SWM(g, "fp64", learned_weights=p)
    R, w = m.learned_weights()
    m.close()
    net = learned.Mlp(params=p)
    x, cell, slot = lw.kite_inputs(g)
    y = net.forward(learned.to_bf16_bits(x))
    Rp, wp = lw.apply_outputs(g, y, cell, slot)
    dR = np.abs(R - Rp).max()
    print(f"learned kite fractions, library vs host pipeline: max diff {dR:.2e}")
    # the features are formed in FP64 by both and rounded to BF16; a value on a
    # BF16 rounding boundary can land on either side
    assert dR < 2e-3
    assert np.median(np.abs(R - Rp)) < 1e-6
    np.testing.assert_allclose(w, lw.trsk_weights(g.nnb, R), rtol=0, atol=1e-15)
    assert np.allclose(R.sum(axis=1), 1.0, atol=1e-14)


@pytest.mark.parametrize("level", [4, 5])
def test_fp64_bitwise_with_the_learned_weights(grid_at, level):
    g = grid_at(level)
    h, u = fields.balanced_state(g, lmax=16, seed=31)
    m = SWM(g, "fp64", learned_weights=_params())
    R, w = m.learned_weights()
    hg, ug = m.ode_rk4(h, u, 600.0, 24)
    assert m.diagnostics()["learned_active"] == 1
    m.close()
    hr, ur = oracle.Oracle(lw.with_weights(g, R, w), 2).run(h, u, 600.0, 24)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_fp32_with_the_learned_weights(grid_at, variant):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=32)
    m = SWM(g, "fp32", learned_weights=_params())
    m.set_tuning(variant=variant)
    R, w = m.learned_weights()
    hg, ug = m.ode_rk4(h, u, 450.0, 48)
    assert m.diagnostics()["learned_active"] == 1
    m.close()
    hr, ur = oracle.Oracle(lw.with_weights(g, R, w), 2).run(h, u, 450.0, 48)
    eh, eu = rel(hg, hr, g.hx_areag), rel(ug, ur, g.ed_leng * g.edhx_leng)
    print(f"variant {variant}: FP32 learned weights vs FP64 oracle h {eh:.2e} u {eu:.2e}")
    assert eh < 1e-6 and eu < 1e-5


@pytest.mark.parametrize("level,dt,days", [(6, 225.0, 2.0), (7, 112.5, 2.0)])
def test_the_trained_network_lowers_the_case2_error(grid_at, level, dt, days):
    """Case 2 (swm.f90:1205-1326) is steady: after `days` the h and u
    departures from the initial state are the scheme's error.  The trained
    network (fitted on levels 5 and 6) must lower both at these levels."""
    if lw.trained_params() is None:
        pytest.skip("no trained parameters in imodel_gb300/data")
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    n = int(round(days * 86400.0 / dt))
    err = {}
    for name, kw in (("plain", {}), ("learned", {"learned_weights": lw.trained_params()})):
        m = SWM(g, "fp32", **kw)
        h1, u1 = m.ode_rk4(h, u, dt, n)
        d = m.diagnostics()
        m.close()
        err[name] = (rel(h1, h, g.hx_areag), rel(u1, u, g.ed_leng * g.edhx_leng))
        if name == "learned":
            assert d["learned_active"] == 1
    print(f"level {level}, {days} days: case-2 error h {err['plain'][0]:.3e} -> "
          f"{err['learned'][0]:.3e}, u {err['plain'][1]:.3e} -> {err['learned'][1]:.3e}")
    assert err["learned"][0] < 0.6 * err["plain"][0]
    assert err["learned"][1] < 0.9 * err["plain"][1]


def test_guard_falls_back_to_plain_trsk(grid_at):
    """A drift bound nothing can meet trips the guard at its first check:
    the interval is stepped again with the plain weights, which then stay
    on; the result equals a plain run bit for bit."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=33)
    m = SWM(g, "fp32", learned_weights=_params(), drift_bound=1e-300)
    m.set_state(h, u)
    m.advance(900.0, 64)
    assert m.diagnostics()["learned_active"] == 0
    hg, ug = m.get_state()
    m.close()
    p = SWM(g, "fp32")
    p.set_state(h, u)
    p.advance(900.0, 64)
    hp, up = p.get_state()
    p.close()
    assert np.array_equal(hg, hp) and np.array_equal(ug, up)


def test_launches_and_refusals(grid_at):
    g = grid_at(3)
    plain = SWM(g, "fp32")
    lw_h = SWM(g, "fp32", learned_weights=_params())
    assert lw_h.launch_count(4) == plain.launch_count(4)
    with pytest.raises(SWMError) as e:
        plain.learned_weights()
    assert e.value.code == _capi.ESTATE
    with pytest.raises(SWMError) as e:
        SWM(g, "fp64", scheme="pxt16", learned_weights=_params())
    assert e.value.code == _capi.EINVAL
    opts = _capi.Opts()
    opts.precision = _capi.FP32
    opts.testcase = 2
    opts.learned = 2
    short = np.zeros(100, dtype=np.float32)
    opts.mlp_weights = short.ctypes.data
    opts.mlp_bytes = short.nbytes
    h = ctypes.c_void_p()
    lib = _capi.swm_lib()
    assert lib.imodel_swm_create(ctypes.byref(g.c_struct()), ctypes.byref(opts),
                                 ctypes.byref(h)) == _capi.EINVAL
    lib.imodel_swm_destroy(h)


def test_error_proxy_measures_the_departure_and_trips_the_guard(grid_at):
    """The guard's error proxy (imodel_swm_opts.error_bound): how far the
    learned weights move plain TRSK's PV flux, ||T_learned - T_plain|| /
    ||Q_plain|| (L2, edge weights l d), measured when the state is set and
    every 256 steps.  It equals the same ratio formed from the two handles'
    tendencies and the oracle's PV flux; a bound below it switches the
    learned weights off at once, and the run then equals a plain run bit
    for bit."""
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=34)
    m = SWM(g, "fp32", learned_weights=_params())
    m.set_state(h, u)
    v0 = m.learned_error_proxy()
    _, tl = m.tendency(h, u)
    p = SWM(g, "fp32")
    _, tp = p.tendency(h, u)
    p.close()
    o = oracle.Oracle(g, 2)
    o.tendency(h, u)
    q = o.field("uhq_perp")
    w = g.ed_leng * g.edhx_leng
    ref = float(np.sqrt(np.sum(w * (tl - tp) ** 2) / np.sum(w * q * q)))
    m.set_state(h, u)
    m.advance(450.0, 300)
    v1 = m.learned_error_proxy()
    assert m.diagnostics()["learned_active"] == 1
    m.close()
    print(f"error proxy of the learned weights: {v0:.4f} at the start (host {ref:.4f}), "
          f"{v1:.4f} after 256 steps")
    assert abs(v0 - ref) <= 1e-3 * ref
    assert 0.001 < v0 < 0.25 and 0.001 < v1 < 0.25 and v1 != v0
    # a bound below the measured departure: off at once, then plain TRSK
    m = SWM(g, "fp32", learned_weights=_params(), error_bound=0.5 * v0)
    m.set_state(h, u)
    assert m.diagnostics()["learned_active"] == 0
    m.advance(450.0, 40)
    hg, ug = m.get_state()
    m.close()
    p = SWM(g, "fp32")
    p.set_state(h, u)
    p.advance(450.0, 40)
    hp, up = p.get_state()
    p.close()
    assert np.array_equal(hg, hp) and np.array_equal(ug, up)


def test_error_proxy_of_the_per_step_network(grid_at):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=35)
    pn = learned.trained_params()
    if pn is None:
        pytest.skip("no trained per-step network in imodel_gb300/data")
    m = SWM(g, "fp32", learned_params=pn)
    m.set_state(h, u)
    v = m.learned_error_proxy()
    m.close()
    print(f"error proxy of the per-step network: {v:.4f}")
    assert 0.0 < v < 0.25
    m = SWM(g, "fp32", learned_params=pn, error_bound=0.5 * v)
    m.set_state(h, u)
    assert m.diagnostics()["learned_active"] == 0
    m.close()
    with pytest.raises(SWMError) as e:
        SWM(g, "fp32").learned_error_proxy()
    assert e.value.code == _capi.ESTATE
    with pytest.raises(SWMError) as e:
        SWM(g, "fp32", learned_params=pn, error_bound=-1.0)
    assert e.value.code == _capi.EINVAL
