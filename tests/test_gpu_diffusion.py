"""Diffusion and hyperdiffusion of the momentum on the GPU
(imodel_swm_set_diffusion): the FP64 path equals the oracle bit for bit,
tendency and RK4 steps; the FP32 variants stay within FP32 round-off; the
terms switch off again."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import fields
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu

# (K2, K4) within the RK4 stability limit at level 5, dt = 450 s; with both on,
# the Laplacian term uses sqrt(K4) (the reference's coefficients), here 3.2e6
CASES = [(1.0e5, 0.0), (0.0, 1.0e14), (1.0e5, 1.0e13)]


@pytest.mark.parametrize("k2,k4", CASES)
def test_fp64_equals_oracle(grid_at, k2, k4):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=6)
    m = SWM(g, "fp64")
    m.set_diffusion(k2, k4)
    o = oracle.Oracle(g, 2, k2=k2, k4=k4)
    mg, ug = m.tendency(h, u)
    mr, ur = o.tendency(h, u)
    assert np.array_equal(mg, mr) and np.array_equal(ug, ur)
    hg, ug = m.ode_rk4(h, u, 600.0, 10)
    hr, ur = o.run(h, u, 600.0, 10)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("k2,k4", CASES)
def test_fp32_close_to_oracle(grid_at, variant, k2, k4):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=7)
    m = SWM(g, "fp32")
    m.set_tuning(variant=variant)
    m.set_diffusion(k2, k4)
    hg, ug = m.ode_rk4(h, u, 450.0, 24)
    hr, ur = oracle.Oracle(g, 2, k2=k2, k4=k4).run(h, u, 450.0, 24)
    w = g.ed_leng * g.edhx_leng
    eh = np.sqrt(np.sum(g.hx_areag * (hg - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
    eu = np.sqrt(np.sum(w * (ug - ur) ** 2) / np.sum(w * ur ** 2))
    assert eh < 1e-6 and eu < 1e-5, (eh, eu)


def test_switching_off_restores_the_plain_step(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=8)
    a = SWM(g, "fp64")
    b = SWM(g, "fp64")
    a.set_diffusion(1.0e5, 1.0e15)
    n0 = a.launch_count(1)
    a.set_diffusion(0.0, 0.0)
    assert a.launch_count(1) < n0
    ha, ua = a.ode_rk4(h, u, 600.0, 5)
    hb, ub = b.ode_rk4(h, u, 600.0, 5)
    assert np.array_equal(ha, hb) and np.array_equal(ua, ub)


FIELD_CASES = [("diam", 1.0e5, 0.0), ("align", 0.0, 1.0e14), ("diam", 1.0e5, 1.0e13)]


def _fields(g, name, k2, k4):
    from imodel_gb300 import difcoef
    f = difcoef.FUNCTIONS[name]
    return (f(g, k2) if k2 else None), (f(g, k4) if k4 else None)


@pytest.mark.parametrize("name,k2,k4", FIELD_CASES)
def test_fp64_coefficient_fields_equal_oracle(grid_at, name, k2, k4):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=14)
    f2, f4 = _fields(g, name, k2, k4)
    m = SWM(g, "fp64")
    m.set_diffusion_fields(f2, f4)
    o = oracle.Oracle(g, 2, k2_hx=f2, k4_hx=f4)
    mg, ug = m.tendency(h, u)
    mr, ur = o.tendency(h, u)
    assert np.array_equal(mg, mr) and np.array_equal(ug, ur)
    hg, ug = m.ode_rk4(h, u, 600.0, 8)
    hr, ur = o.run(h, u, 600.0, 8)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_fp32_coefficient_fields_close_to_oracle(grid_at, variant):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=15)
    f2, f4 = _fields(g, "diam", 1.0e5, 1.0e13)
    m = SWM(g, "fp32")
    m.set_tuning(variant=variant)
    m.set_diffusion_fields(f2, f4)
    hg, ug = m.ode_rk4(h, u, 450.0, 24)
    hr, ur = oracle.Oracle(g, 2, k2_hx=f2, k4_hx=f4).run(h, u, 450.0, 24)
    w = g.ed_leng * g.edhx_leng
    eh = np.sqrt(np.sum(g.hx_areag * (hg - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
    eu = np.sqrt(np.sum(w * (ug - ur) ** 2) / np.sum(w * ur ** 2))
    assert eh < 1e-6 and eu < 1e-5, (eh, eu)


def test_coefficient_field_refusals(grid_at):
    from imodel_gb300 import _capi
    from imodel_gb300.swm import SWMError
    g = grid_at(3)
    m = SWM(g, "fp64")
    f = np.full(g.nv, 1.0e5)
    f[7] = -1.0
    with pytest.raises(SWMError) as ei:
        m.set_diffusion_fields(f, None)
    assert ei.value.code == _capi.EINVAL
    with pytest.raises(ValueError):
        m.set_diffusion_fields(np.ones(5), None)
