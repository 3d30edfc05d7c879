"""Edge cases of the step on the GPU: the smallest meshes (icos level 0 is 12
pentagons, 30 edges and 20 triangles: fewer entities than a warp, a network
tile or a 16-bit record warp), the learned correction on them, an ensemble
with an odd member count, and the call-order and argument errors of the C
ABI."""
import ctypes

import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, fields, learned, swm
from imodel_gb300.swm import SWM, Ensemble, SWMError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("level", [0, 1])
def test_tiny_meshes_fp64_bitwise(grid_at, level):
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    m = SWM(g, "fp64")
    o = oracle.Oracle(g, 2)
    mg, ug = m.tendency(h, u)
    mr, ur = o.tendency(h, u)
    assert np.array_equal(mg, mr) and np.array_equal(ug, ur)
    hg, ug = m.ode_rk4(h, u, 3600.0, 3)
    hr, ur = o.run(h, u, 3600.0, 3)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("level", [0, 1])
def test_tiny_meshes_fp32(grid_at, level, variant):
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    m = SWM(g, "fp32")
    m.set_tuning(variant=variant)
    hg, ug = m.ode_rk4(h, u, 3600.0, 3)
    hr, ur = oracle.Oracle(g, 2).run(h, u, 3600.0, 3)
    assert np.max(np.abs(hg - hr)) < 1e-6 * np.max(np.abs(hr))
    assert np.max(np.abs(ug - ur)) < 1e-5 * np.max(np.abs(ur))


def test_learned_on_tiny_mesh(grid_at):
    """One partial network tile (30 edges of 128 rows): a zero network still
    equals the plain step bit for bit, the trained one stays finite."""
    from oracle import mlp_oracle as mo
    g = grid_at(0)
    h, u = swm.initialize_fields_tc2(g)
    a = SWM(g, "fp32", learned_params=np.zeros(mo.NPARAM, dtype=np.float32))
    b = SWM(g, "fp32")
    b.set_tuning(variant=1)
    ha, ua = a.ode_rk4(h, u, 3600.0, 4)
    hb, ub = b.ode_rk4(h, u, 3600.0, 4)
    assert np.array_equal(ha, hb) and np.array_equal(ua, ub)
    c = SWM(g, "fp32", learned_params=learned.trained_params())
    hc, uc = c.ode_rk4(h, u, 3600.0, 4)
    assert np.all(np.isfinite(hc)) and np.all(np.isfinite(uc))


def test_ensemble_odd_member_count(grid_at):
    g = grid_at(2)
    states = [fields.balanced_state(g, lmax=6, seed=s) for s in (1, 2, 3)]
    ens = Ensemble([g], [3])
    for m, (h, u) in enumerate(states):
        ens.set_state(0, m, h, u)
    ens.advance([900.0], [4])
    for m, (h, u) in enumerate(states):
        he, ue = ens.get_state(0, m)
        hr, ur = oracle.Oracle(g, 2).run(h, u, 900.0, 4)
        assert np.max(np.abs(he - hr)) < 1e-6 * np.max(np.abs(hr))
        assert np.max(np.abs(ue - ur)) < 1e-5 * np.max(np.abs(ur))


def test_call_order_and_arguments(grid_at):
    g = grid_at(2)
    h, u = swm.initialize_fields_tc2(g)
    m = SWM(g, "fp32")
    with pytest.raises(SWMError) as ei:   # no state yet
        m.advance(600.0, 1)
    assert ei.value.code == _capi.ESTATE
    with pytest.raises(SWMError) as ei:
        m.get_state()
    assert ei.value.code == _capi.ESTATE
    m.set_state(h, u)
    h0, u0 = m.get_state()
    m.advance(600.0, 0)                   # zero steps: nothing changes
    h1, u1 = m.get_state()
    assert np.array_equal(h0, h1) and np.array_equal(u0, u1)
    for dt, n in ((600.0, -1), (float("nan"), 1), (float("inf"), 1)):
        with pytest.raises(SWMError) as ei:
            m.advance(dt, n)
        assert ei.value.code == _capi.EINVAL
    for k2, k4 in ((-1.0, 0.0), (0.0, float("nan"))):
        with pytest.raises(SWMError) as ei:
            m.set_diffusion(k2, k4)
        assert ei.value.code == _capi.EINVAL
    with pytest.raises(SWMError) as ei:
        m.set_tuning(variant=5)
    assert ei.value.code == _capi.EINVAL
    with pytest.raises(SWMError) as ei:
        m.set_tuning(variant=1, bs_cell=96)
    assert ei.value.code == _capi.EINVAL
    # the learned correction needs the FP32 path and its parameter count
    with pytest.raises(SWMError) as ei:
        SWM(g, "fp64", learned_params=learned.trained_params())
    assert ei.value.code == _capi.EINVAL
    with pytest.raises(SWMError) as ei:
        SWM(g, "fp32", learned_params=np.zeros(10, dtype=np.float32))
    assert ei.value.code == _capi.EINVAL
    # still usable after the refusals
    h2, u2 = m.ode_rk4(h, u, 600.0, 2)
    assert np.all(np.isfinite(h2)) and np.all(np.isfinite(u2))
    assert m.lib.imodel_swm_step(m.handle, None, None, 600.0, 1) == _capi.EINVAL
    assert ctypes.c_void_p(m.handle.value).value is not None
