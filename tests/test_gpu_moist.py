"""The moist shallow-water model on the GPU (include/imodel_moist.h) equals
the CPU oracle bit for bit: FP64 in the reference's operation order, the
tracers, the thermal momentum source and the water sources included.  The
FP32 handle stays within FP32 round-off of the FP64 one and conserves mass
and total water."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, moist
from imodel_gb300.swm import SWMError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,level,dt,n,adv", [
    (1, 4, 1800.0, 48, "trsk"), (2, 4, 900.0, 48, "trsk"), (3, 4, 600.0, 48, "trsk"),
    (3, 5, 300.0, 24, "trsk"), (4, 4, 600.0, 48, "trsk"), (5, 5, 300.0, 24, "trsk"),
    (1, 4, 1800.0, 48, "upw1"), (3, 4, 600.0, 48, "upw1"), (4, 5, 300.0, 24, "upw1")])
def test_fp64_equals_oracle(grid_at, case, level, dt, n, adv):
    g = grid_at(level)
    f = moist.moist_fields(g, case)
    m = moist.Moist(g, case, f, advection=adv)
    m.set_state(f)
    m.advance(dt, n // 2)
    m.advance(dt, n - n // 2)
    s = m.get_state()
    m.close()
    r = oracle.MoistOracle(g, case, f, advection=adv).run(f, dt, n)
    for k in moist.FIELDS:
        assert np.array_equal(s[k], r[k]), (k, np.max(np.abs(s[k] - r[k])))


@pytest.mark.parametrize("adv", ["trsk", "upw1"])
def test_fp64_long_jet_run_equals_oracle(grid_at, adv):
    """240 steps (20 hours) of the moist Galewsky jet at level 5, in chunks
    of the graph-replayed step: still bit-equal to the oracle."""
    g = grid_at(5)
    f = moist.moist_fields(g, 4)
    m = moist.Moist(g, 4, f, advection=adv)
    m.set_state(f)
    for _ in range(3):
        m.advance(300.0, 80)
    s = m.get_state()
    m.close()
    r = oracle.MoistOracle(g, 4, f, advection=adv).run(f, 300.0, 240)
    for k in moist.FIELDS:
        assert np.array_equal(s[k], r[k]), (k, np.max(np.abs(s[k] - r[k])))


def test_call_order_and_arguments(grid_at):
    g = grid_at(3)
    f = moist.moist_fields(g, 2)
    m = moist.Moist(g, 2, f)
    with pytest.raises(SWMError) as e:
        m.advance(900.0, 1)
    assert e.value.code == _capi.ESTATE
    m.set_state(f)
    with pytest.raises(SWMError) as e:
        m.advance(-1.0, 1)
    assert e.value.code == _capi.EINVAL
    m.close()
    with pytest.raises(SWMError) as e:
        moist.Moist(g, 9, f)
    assert e.value.code == _capi.EINVAL
    # an advection method that is not built is refused at create
    import ctypes
    o = _capi.MoistOpts()
    o.testcase = 1
    th = np.zeros(g.nv)
    o.theta = _capi.as_f64p(th)
    o.advection = 5
    h = ctypes.c_void_p()
    lib = _capi.swm_lib()
    assert lib.imodel_moist_create(ctypes.byref(g.c_struct()), ctypes.byref(o),
                                   ctypes.byref(h)) == _capi.EINVAL
    lib.imodel_moist_destroy(h)


def _rel_l2(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / max(np.sum(w * b * b), 1e-300)))


# (case, level, dt, steps, advection): FP32 against FP64 after the same
# steps; bounds about ten times the largest differences measured on a GB300
# (h 6e-8, u 5e-7, h theta 6e-7, h qv 2e-7, tracer 3e-7; the cloud and rain
# water, whose sources switch on thresholds, 7e-4 and 5e-5)
FP32_BOUND = {"h": 1e-6, "u": 5e-6, "htheta": 1e-5, "hqv": 5e-6, "hqc": 1e-2, "hqr": 1e-3,
              "htracer": 5e-6}
FP32_CASES = [(1, 5, 900.0, 48, "trsk"), (2, 5, 600.0, 72, "trsk"), (3, 5, 300.0, 96, "trsk"),
              (4, 5, 300.0, 96, "trsk"), (5, 5, 300.0, 96, "trsk"), (3, 5, 300.0, 96, "upw1"),
              (4, 5, 300.0, 96, "upw1")]


@pytest.mark.parametrize("case,level,dt,n,adv", FP32_CASES)
def test_fp32_against_fp64(grid_at, case, level, dt, n, adv):
    g = grid_at(level)
    f = moist.moist_fields(g, case)
    out = {}
    for prec in ("fp64", "fp32"):
        m = moist.Moist(g, case, f, advection=adv, precision=prec)
        m.set_state(f)
        m.advance(dt, n)
        out[prec] = m.get_state()
        m.close()
    a, b = out["fp32"], out["fp64"]
    wc = g.hx_areag
    we = g.ed_leng * g.edhx_leng
    d = {k: _rel_l2(a[k], b[k], we if k == "u" else wc) for k in moist.FIELDS
         if np.any(b[k] != 0)}
    print(f"case {case} {adv}: FP32 vs FP64 rel L2 " +
          ", ".join(f"{k} {v:.1e}" for k, v in d.items()))
    for k, v in d.items():
        assert np.all(np.isfinite(a[k])), k
        assert v < FP32_BOUND[k], (k, v)
    # the sources move water between its three forms only, and the flux
    # form conserves each total: total water and mass to FP32 round-off
    w0 = np.sum(wc * (f["hqv"] + f["hqc"] + f["hqr"]))
    w1 = np.sum(wc * (a["hqv"] + a["hqc"] + a["hqr"]))
    if w0 != 0:
        assert abs(w1 - w0) / abs(w0) < 1e-5, (w0, w1)
    m0, m1 = np.sum(wc * f["h"]), np.sum(wc * a["h"])
    assert abs(m1 - m0) / abs(m0) < 1e-6, (m0, m1)


def test_fp32_precision_argument(grid_at):
    g = grid_at(3)
    f = moist.moist_fields(g, 2)
    with pytest.raises(ValueError):
        moist.Moist(g, 2, f, precision="fp16")
    import ctypes
    o = _capi.MoistOpts()
    o.testcase = 2
    th = np.ascontiguousarray(f["theta"])
    o.theta = _capi.as_f64p(th)
    o.precision = 7
    h = ctypes.c_void_p()
    lib = _capi.swm_lib()
    assert lib.imodel_moist_create(ctypes.byref(g.c_struct()), ctypes.byref(o),
                                   ctypes.byref(h)) == _capi.EINVAL
    lib.imodel_moist_destroy(h)
