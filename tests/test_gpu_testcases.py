"""The step from the states of test cases 1, 5, 6 and 21: the FP64 GPU path
equals the oracle bit for bit (case 5 with its topography, case 1 with the
momentum equation and PV off), the FP32 path stays within FP32 round-off."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import testcases as tc
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,dt", [(1, 900.0), (5, 600.0), (6, 600.0), (21, 600.0), (56, 300.0),
                                     (57, 1800.0)])
def test_fp64_equals_oracle(grid_at, case, dt):
    g = grid_at(5)
    h, u, bt = tc.initialize_fields(g, case)
    m = SWM(g, "fp64", testcase=case, bt=bt)
    hg, ug = m.ode_rk4(h, u, dt, 12)
    hr, ur = oracle.Oracle(g, case, bt=bt).run(h, u, dt, 12)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("case,dt", [(1, 900.0), (5, 600.0), (6, 600.0), (21, 600.0), (56, 300.0),
                                     (57, 1800.0)])
def test_fp32_close_to_oracle(grid_at, case, dt):
    g = grid_at(5)
    h, u, bt = tc.initialize_fields(g, case)
    m = SWM(g, "fp32", testcase=case, bt=bt)
    hg, ug = m.ode_rk4(h, u, dt, 48)
    hr, ur = oracle.Oracle(g, case, bt=bt).run(h, u, dt, 48)
    eh = np.sqrt(np.sum(g.hx_areag * (hg - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
    w = g.ed_leng * g.edhx_leng
    eu = np.sqrt(np.sum(w * (ug - ur) ** 2) / np.sum(w * ur ** 2))
    print(f"case {case}: FP32 vs oracle after 48 steps, rel L2 h {eh:.2e} u {eu:.2e}")
    assert eh < 1e-6 and eu < 1e-5
