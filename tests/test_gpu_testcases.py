"""The step from the states of the reference's test cases: the FP64 GPU
path equals the oracle bit for bit (cases with topography, case 1 with the
momentum equation and PV off, the f-sphere cases with their constant f),
the FP32 path stays within FP32 round-off."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import testcases as tc
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu


CASES = [(1, 900.0), (5, 600.0), (6, 600.0), (21, 600.0), (56, 300.0), (57, 1800.0),
         (32, 600.0), (33, 600.0), (40, 120.0), (41, 60.0), (42, 60.0), (43, 600.0),
         (52, 600.0), (53, 600.0)]


def _fields(g, case):
    if case == 51:
        return tc.tc51(g, hollgw=50.0)
    return tc.initialize_fields(g, case)


@pytest.mark.parametrize("case,dt", CASES + [(51, 600.0)])
def test_fp64_equals_oracle(grid_at, case, dt):
    g = grid_at(5)
    h, u, bt = _fields(g, case)
    opts = tc.case_options(case)
    m = SWM(g, "fp64", bt=bt, **opts)
    hg, ug = m.ode_rk4(h, u, dt, 12)
    hr, ur = oracle.Oracle(g, bt=bt, **opts).run(h, u, dt, 12)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)


@pytest.mark.parametrize("case,dt", [c for c in CASES if c[0] not in (32, 33)])
def test_fp32_close_to_oracle(grid_at, case, dt):
    g = grid_at(5)
    h, u, bt = _fields(g, case)
    opts = tc.case_options(case)
    m = SWM(g, "fp32", bt=bt, **opts)
    hg, ug = m.ode_rk4(h, u, dt, 48)
    hr, ur = oracle.Oracle(g, bt=bt, **opts).run(h, u, dt, 48)
    eh = np.sqrt(np.sum(g.hx_areag * (hg - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
    w = g.ed_leng * g.edhx_leng
    eu = np.sqrt(np.sum(w * (ug - ur) ** 2) / np.sum(w * ur ** 2))
    print(f"case {case}: FP32 vs oracle after 48 steps, rel L2 h {eh:.2e} u {eu:.2e}")
    assert eh < 1e-6 and eu < 1e-5
