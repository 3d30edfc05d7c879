"""The anticipated potential vorticity method on the GPU
(imodel_swm_set_apvm): the FP64 step equals the oracle bit for bit,
tendency and RK4 steps, alone and with diffusion; the FP32 step (the stencil
variant and both cell-centred variants) stays within FP32 round-off of it;
it costs one launch per stage in variant 0, two in the others; it switches
off again; it runs together with the per-step learned correction."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, fields, swm
from imodel_gb300.swm import SWM, SWMError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("level,state", [(3, "tc2"), (4, "balanced"), (5, "balanced")])
def test_fp64_equals_oracle(grid_at, level, state):
    g = grid_at(level)
    if state == "tc2":
        h, u = swm.initialize_fields_tc2(g)
    else:
        h, u = fields.balanced_state(g, lmax=12, seed=11)
    dt = 600.0
    m = SWM(g, "fp64")
    m.set_apvm(0.5, dt)
    o = oracle.Oracle(g, 2, pvspar=0.5, dt=dt)
    mg, ug = m.tendency(h, u)
    mr, ur = o.tendency(h, u)
    assert np.array_equal(mg, mr) and np.array_equal(ug, ur)
    hg, ug = m.ode_rk4(h, u, dt, 8)
    hr, ur = o.run(h, u, dt, 8)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
    # the correction changed the step
    hp, up = oracle.Oracle(g, 2).run(h, u, dt, 8)
    assert not np.array_equal(up, ur)


def test_fp64_with_diffusion_equals_oracle(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=12)
    m = SWM(g, "fp64")
    m.set_apvm(1.0, 600.0)
    m.set_diffusion(1.0e5, 1.0e13)
    o = oracle.Oracle(g, 2, k2=1.0e5, k4=1.0e13, pvspar=1.0, dt=600.0)
    hg, ug = m.ode_rk4(h, u, 600.0, 6)
    hr, ur = o.run(h, u, 600.0, 6)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


def test_launch_count_and_switching_off(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=13)
    a = SWM(g, "fp64")
    n0 = a.launch_count(1)
    a.set_apvm(0.5, 600.0)
    assert a.launch_count(1) == n0 + 8      # edge gradients, reconstructions
    a.set_apvm(0.0, 600.0)
    assert a.launch_count(1) == n0
    ha, ua = a.ode_rk4(h, u, 600.0, 4)
    hb, ub = SWM(g, "fp64").ode_rk4(h, u, 600.0, 4)
    assert np.array_equal(ha, hb) and np.array_equal(ua, ub)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_fp32_close_to_oracle(grid_at, variant):
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=7)
    m = SWM(g, "fp32")
    m.set_apvm(0.5, 450.0)
    m.set_tuning(variant=variant)
    # variant 0: four kernels and the reconstructions; 1 and 2: three, the
    # reconstructions and the edge pre-pass
    assert m.launch_count(1) == 4 * 5
    hg, ug = m.ode_rk4(h, u, 450.0, 24)
    hr, ur = oracle.Oracle(g, 2, pvspar=0.5, dt=450.0).run(h, u, 450.0, 24)
    hp, up = oracle.Oracle(g, 2).run(h, u, 450.0, 24)
    w = g.ed_leng * g.edhx_leng
    rel_h = lambda a, b: np.sqrt(np.sum(g.hx_areag * (a - b) ** 2) / np.sum(g.hx_areag * b ** 2))
    rel_u = lambda a, b: np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b ** 2))
    eh, eu = rel_h(hg, hr), rel_u(ug, ur)
    print(f"variant {variant}: FP32 + APVM vs the oracle: h {eh:.2e}, u {eu:.2e}")
    assert eh < 1e-6 and eu < 1e-5, (eh, eu)
    # the correction itself is far above that (1.4e-4 in h, 3.9e-3 in u)
    assert rel_h(hg, hp) > 50 * eh and rel_u(ug, up) > 50 * eu


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_fp32_with_diffusion_close_to_oracle(grid_at, variant):
    """APVM with Laplacian and hyperdiffusion on, in each FP32 variant."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=12)
    m = SWM(g, "fp32")
    m.set_apvm(1.0, 600.0)
    m.set_diffusion(1.0e5, 1.0e13)
    m.set_tuning(variant=variant)
    hg, ug = m.ode_rk4(h, u, 600.0, 12)
    hr, ur = oracle.Oracle(g, 2, k2=1.0e5, k4=1.0e13, pvspar=1.0, dt=600.0).run(h, u, 600.0, 12)
    w = g.ed_leng * g.edhx_leng
    eh = np.sqrt(np.sum(g.hx_areag * (hg - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
    eu = np.sqrt(np.sum(w * (ug - ur) ** 2) / np.sum(w * ur ** 2))
    print(f"variant {variant}: FP32 + APVM + diffusion vs the oracle: h {eh:.2e}, u {eu:.2e}")
    assert eh < 1e-6 and eu < 1e-5, (eh, eu)


def test_apvm_with_the_per_step_learned_correction(grid_at):
    """APVM and the per-step network correction (cell-centred variants) run
    together: the step differs from either alone and from plain FP32 by
    about the sum of the two changes."""
    from imodel_gb300 import learned
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=16, seed=9)
    dt, n = 450.0, 24
    w = g.ed_leng * g.edhx_leng
    rel_u = lambda a, b: np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b ** 2))
    runs = {}
    for name, net, pv in (("plain", False, 0.0), ("apvm", False, 0.5), ("net", True, 0.0),
                          ("both", True, 0.5)):
        m = SWM(g, "fp32", learned_params=learned.trained_params()) if net else SWM(g, "fp32")
        if pv:
            m.set_apvm(pv, dt)
        runs[name] = m.ode_rk4(h, u, dt, n)
        m.close()
    up = runs["plain"][1]
    da, dn, db = (rel_u(runs[k][1], up) for k in ("apvm", "net", "both"))
    print(f"u vs plain FP32: apvm {da:.2e}, network {dn:.2e}, both {db:.2e}")
    assert all(np.all(np.isfinite(x)) for r in runs.values() for x in r)
    assert da > 1e-5 and dn > 1e-5
    assert rel_u(runs["both"][1], runs["apvm"][1]) > 0.3 * dn
    assert rel_u(runs["both"][1], runs["net"][1]) > 0.3 * da


def test_refusals(grid_at):
    g = grid_at(3)
    m = SWM(g, "fp32")
    m.set_apvm(0.5, 600.0)
    for v in (1, 2, 0):                 # every variant runs APVM
        m.set_tuning(variant=v)
    d = SWM(g, "fp64")
    for pv, dt in ((-0.5, 600.0), (float("nan"), 600.0), (0.5, 0.0), (0.5, float("inf"))):
        with pytest.raises(SWMError) as ei:
            d.set_apvm(pv, dt)
        assert ei.value.code == _capi.EINVAL


@pytest.mark.parametrize("fail_at", [1, 2, 3])
def test_failed_allocation_leaves_apvm_off(grid_at, fail_at):
    """An allocation that fails inside set_apvm (injected on the host) returns
    ENOMEM and leaves APVM off: the next steps equal the plain oracle's, and a
    later set_apvm completes the buffers and equals the APVM oracle."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=14)
    dt = 600.0
    m = SWM(g, "fp64")
    lib = _capi.swm_lib()
    assert lib.imodel_swm_test_fail_alloc(fail_at) == 0
    try:
        with pytest.raises(SWMError) as e:
            m.set_apvm(0.5, dt)
        assert e.value.code == _capi.ENOMEM
    finally:
        lib.imodel_swm_test_fail_alloc(0)
    hg, ug = m.ode_rk4(h, u, dt, 3)
    hr, ur = oracle.Oracle(g, 2).run(h, u, dt, 3)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
    m.set_apvm(0.5, dt)
    hg, ug = m.ode_rk4(h, u, dt, 3)
    hr, ur = oracle.Oracle(g, 2, pvspar=0.5, dt=dt).run(h, u, dt, 3)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


def test_failed_allocation_leaves_diffusion_off(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=15)
    dt = 600.0
    m = SWM(g, "fp64")
    lib = _capi.swm_lib()
    assert lib.imodel_swm_test_fail_alloc(4) == 0
    try:
        with pytest.raises(SWMError) as e:
            m.set_diffusion(1.0e5, 0.0)
        assert e.value.code == _capi.ENOMEM
    finally:
        lib.imodel_swm_test_fail_alloc(0)
    hg, ug = m.ode_rk4(h, u, dt, 2)
    hr, ur = oracle.Oracle(g, 2).run(h, u, dt, 2)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
    m.set_diffusion(1.0e5, 0.0)
    hg, ug = m.ode_rk4(h, u, dt, 2)
    hr, ur = oracle.Oracle(g, 2, k2=1.0e5).run(h, u, dt, 2)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
