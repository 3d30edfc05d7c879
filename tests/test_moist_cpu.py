"""The moist shallow-water model's oracle (moist_swm.f90, advmtd = "trsk",
RK4) against the model's own known answers: case 1 advects the tracer alone
and conserves it; case 2 is a steady balanced moist flow, so its error after
a day falls with resolution; water (h qv + h qc + h qr), mass and the tracer
are conserved to round-off, since the sources only exchange water between
the species and every tracer is advected in flux form."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import moist, testcases


def _rel(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b * b)))


def test_case1_advects_the_tracer_alone(grid_at):
    g = grid_at(3)
    f = moist.moist_fields(g, 1)
    s = oracle.MoistOracle(g, 1, f).run(f, 1800.0, 96)
    for k in ("h", "u", "htheta", "hqv", "hqc", "hqr"):
        assert np.array_equal(s[k], f[k]), k
    w = g.hx_areag
    assert _rel(s["htracer"], f["htracer"], w) > 1e-2       # it moved
    assert abs(np.sum(w * s["htracer"]) / np.sum(w * f["htracer"]) - 1.0) < 1e-14


def test_case2_steady_state_converges(grid_at):
    errs = []
    for L, dt in ((3, 1800.0), (4, 900.0), (5, 450.0)):
        g = grid_at(L)
        f = moist.moist_fields(g, 2)
        s = oracle.MoistOracle(g, 2, f).run(f, dt, int(86400.0 / dt))
        errs.append(_rel(s["h"], f["h"], g.hx_areag))
    assert errs[0] > 2.3 * errs[1] > 2.3 * 2.3 * errs[2], errs
    assert errs[2] < 5e-4


@pytest.mark.parametrize("case", [2, 3, 4, 5])
def test_water_mass_and_tracer_are_conserved(grid_at, case):
    g = grid_at(4)
    f = moist.moist_fields(g, case)
    s = oracle.MoistOracle(g, case, f).run(f, 600.0, 48)
    w = g.hx_areag
    water = lambda x: np.sum(w * (x["hqv"] + x["hqc"] + x["hqr"]))  # noqa: E731
    assert abs(water(s) / water(f) - 1.0) < 1e-14
    assert abs(np.sum(w * s["h"]) / np.sum(w * f["h"]) - 1.0) < 1e-14
    assert np.sum(w * s["hqc"]) > 0.0            # cloud formed from the vapour
    if case >= 3:
        assert np.array_equal(s["htracer"], f["htracer"])   # not advected in cases 3-5


def test_initial_states(grid_at):
    g = grid_at(4)
    f2 = moist.moist_fields(g, 2)
    # case 2 starts saturated: qv = qsat(theta, h, b) with the case's q0
    np.testing.assert_allclose(f2["qv"], moist.qsat(f2["theta"], f2["h"], f2["bt"], f2["q0"]),
                               rtol=1e-14)
    assert abs(f2["qv"].max() - 0.02) < 1e-15
    f3 = moist.moist_fields(g, 3)
    k = int(np.argmax(f3["bt"]))
    assert 1000.0 < f3["bt"][k] <= 2000.0
    # the cone stands at (120, 30) degrees
    assert abs(np.degrees(g.v_lon[k]) - 120.0) < 8.0 and abs(np.degrees(g.v_lat[k]) - 30.0) < 8.0
    assert abs(f3["qv"].max() - 0.02) < 1e-15
    for case, base, lat2, lonc in ((4, 22, 45.0, 167.4 - 120.0), (5, 52, -25.0, 167.4)):
        f = moist.moist_fields(g, case)
        h0, u0, _ = testcases.galewsky(g, base)
        assert np.array_equal(f["u"], u0)              # the barotropic jet
        bump = f["h"] - h0                   # the 120 m cos(lat) bump, where stated
        k = int(np.argmax(bump))
        peak = 120.0 * np.cos(np.radians(lat2))
        assert 0.85 * peak < bump[k] <= peak
        assert abs(np.degrees(g.v_lat[k]) - lat2) < 6.0
        assert abs(np.degrees(g.v_lon[k]) - lonc) < 8.0
        assert abs(f["qv"].max() - 0.02) < 1e-15
        np.testing.assert_allclose(f["qv"], moist.qsat(f["theta"], f["h"], 0.0, 0.98 * f["q0"]),
                                   rtol=1e-14)
    with pytest.raises(ValueError):
        moist.moist_fields(g, 7)


def test_upwind_advection_is_positive_and_conservative(grid_at):
    """advmtd = "upw1" (div_hx_upw1, highorder.f90:5094-5139): the upwind
    flux keeps case 1's tracer positive where the centred scheme undershoots,
    spreads it more, and conserves it to round-off, as a flux form must."""
    g = grid_at(4)
    f = moist.moist_fields(g, 1)
    w = g.hx_areag
    out = {}
    for adv in ("trsk", "upw1"):
        s = oracle.MoistOracle(g, 1, f, advection=adv).run(f, 1800.0, 96)
        out[adv] = s["htracer"] / s["h"]
        assert abs(np.sum(w * s["htracer"]) / np.sum(w * f["htracer"]) - 1.0) < 1e-14
    assert out["trsk"].min() < -1e-3 < 0.0 <= out["upw1"].min()
    assert out["upw1"].max() < 0.8 * out["trsk"].max()
    with pytest.raises(ValueError):
        oracle.MoistOracle(g, 1, f, advection="og4")
