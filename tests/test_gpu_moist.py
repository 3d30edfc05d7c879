"""The moist shallow-water model on the GPU (include/imodel_moist.h) equals
the CPU oracle bit for bit: FP64 in the reference's operation order, the
tracers, the thermal momentum source and the water sources included."""
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
