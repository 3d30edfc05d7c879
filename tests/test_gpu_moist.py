"""The moist shallow-water model on the GPU (include/imodel_moist.h) equals
the CPU oracle bit for bit: FP64 in the reference's operation order, the
tracers, the thermal momentum source and the water sources included."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, moist
from imodel_gb300.swm import SWMError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,level,dt,n", [(1, 4, 1800.0, 48), (2, 4, 900.0, 48),
                                            (3, 4, 600.0, 48), (3, 5, 300.0, 24)])
def test_fp64_equals_oracle(grid_at, case, level, dt, n):
    g = grid_at(level)
    f = moist.moist_fields(g, case)
    m = moist.Moist(g, case, f)
    m.set_state(f)
    m.advance(dt, n // 2)
    m.advance(dt, n - n // 2)
    s = m.get_state()
    m.close()
    r = oracle.MoistOracle(g, case, f).run(f, dt, n)
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
