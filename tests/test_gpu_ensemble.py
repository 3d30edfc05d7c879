"""Batched ensembles in one persistent launch against single runs.

Every member of every grid must equal the single-run FP32 path (cell-centred
variant) started from the same state, bit for bit: the ensemble kernel runs
the same per-entity code with the members interleaved.
"""
import numpy as np
import pytest

from imodel_gb300 import fields, swm
from imodel_gb300.swm import SWM, Ensemble

pytestmark = pytest.mark.gpu


def _states(g, seeds, lmax):
    return [fields.balanced_state(g, lmax=lmax, seed=s) for s in seeds]


def test_ensemble_members_equal_single_runs(grid_at):
    g4, g3 = grid_at(4), grid_at(3)
    s4 = _states(g4, [0, 1, 2], 16)
    s3 = _states(g3, [100, 101], 12)
    ens = Ensemble([g4, g3], [3, 2])
    for m, (h, u) in enumerate(s4):
        ens.set_state(0, m, h, u)
    for m, (h, u) in enumerate(s3):
        ens.set_state(1, m, h, u)
    dts, steps = [900.0, 1800.0], [24, 11]
    ens.advance(dts, steps)
    for k, (g, states) in enumerate([(g4, s4), (g3, s3)]):
        # the single runs use the h_ref of the grid's first member, as the
        # ensemble does (same sequential sums as the library)
        s = a = 0.0
        for ai, hi in zip(g.hx_areag.tolist(), states[0][0].tolist()):
            a += ai
            s += ai * hi
        h_ref = float(np.float32(s / a))
        for m, (h, u) in enumerate(states):
            single = SWM(g, "fp32", h_ref=h_ref)
            single.set_tuning(variant=1)
            hs, us = single.ode_rk4(h, u, dts[k], steps[k])
            he, ue = ens.get_state(k, m)
            assert np.array_equal(he, hs), (k, m, np.max(np.abs(he - hs)))
            assert np.array_equal(ue, us), (k, m, np.max(np.abs(ue - us)))
    ens.close()


def test_ensemble_tune_keeps_state(grid_at):
    g = grid_at(4)
    states = _states(g, [5, 6], 16)
    ens = Ensemble([g], [2])
    for m, (h, u) in enumerate(states):
        ens.set_state(0, m, h, u)
    before = [ens.get_state(0, m) for m in range(2)]
    choice = ens.tune([900.0], 2)
    assert choice["block"] in (128, 256, 512) and choice["blocks_per_sm"] >= 1
    assert choice["variant"] in (0, 1)
    after = [ens.get_state(0, m) for m in range(2)]
    for (hb, ub), (ha, ua) in zip(before, after):
        assert np.array_equal(hb, ha) and np.array_equal(ub, ua)
    ens.close()


def test_ensemble_blowup_status(grid_at):
    g = grid_at(3)
    h, u = swm.initialize_fields_tc2(g)
    u = u.copy()
    u[7] = np.inf
    ens = Ensemble([g], [1])
    ens.set_state(0, 0, h, u)
    ens.advance([1800.0], [1])
    with pytest.raises(swm.SWMError) as ei:
        ens.get_state(0, 0)
    assert ei.value.code == 3
    ens.close()


def test_ensemble_barrier_timeout_status(grid_at):
    """The persistent launch's grid-wide barriers wait a bounded time: when
    one block never arrives (the test hook makes block 0 leave before its
    first barrier) the others give up after a short wait, the advance reports
    the timeout as a status, and the ensemble still works afterwards."""
    from imodel_gb300 import _capi
    g = grid_at(3)
    states = _states(g, [7, 8], 8)
    ens = Ensemble([g], [2])
    for m, (h, u) in enumerate(states):
        ens.set_state(0, m, h, u)
    lib = _capi.swm_lib()
    assert lib.imodel_swm_ensemble_test_stall(ens._handle, 0, 1 << 14) == 0
    with pytest.raises(swm.SWMError) as ei:
        ens.advance([1800.0], [3])
    assert ei.value.code == _capi.ECUDA and "barrier" in str(ei.value)
    # usable again: the same steps from the same states match a fresh ensemble
    for m, (h, u) in enumerate(states):
        ens.set_state(0, m, h, u)
    ens.advance([1800.0], [3])
    fresh = Ensemble([g], [2])
    for m, (h, u) in enumerate(states):
        fresh.set_state(0, m, h, u)
    fresh.advance([1800.0], [3])
    for m in range(2):
        a, b = ens.get_state(0, m), fresh.get_state(0, m)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    ens.close()
    fresh.close()


def test_ensemble_with_the_learned_trsk_weights(grid_at):
    """The headline method in an ensemble: the learned TRSK weights are a
    corrected mesh, so an ensemble on the weights a learned-weights handle
    exports (imodel_swm_learned_weights) steps every member as that handle
    steps it, bit for bit."""
    from imodel_gb300 import learned, learned_weights as lw
    g = grid_at(4)
    p = lw.trained_params()
    if p is None:
        p = learned.init_params(7)
    probe = SWM(g, "fp32", learned_weights=p)
    R, w = probe.learned_weights()
    probe.close()
    g2 = lw.with_weights(g, R, w)
    states = _states(g, [7, 8], 16)
    ens = Ensemble([g2], [2])
    for m, (h, u) in enumerate(states):
        ens.set_state(0, m, h, u)
    ens.advance([900.0], [24])
    s = a = 0.0
    for ai, hi in zip(g.hx_areag.tolist(), states[0][0].tolist()):
        a += ai
        s += ai * hi
    h_ref = float(np.float32(s / a))
    for m, (h, u) in enumerate(states):
        single = SWM(g, "fp32", h_ref=h_ref, learned_weights=p)
        single.set_tuning(variant=1)
        hs, us = single.ode_rk4(h, u, 900.0, 24)
        assert single.diagnostics()["learned_active"] == 1
        single.close()
        he, ue = ens.get_state(0, m)
        assert np.array_equal(he, hs) and np.array_equal(ue, us), m
    ens.close()
