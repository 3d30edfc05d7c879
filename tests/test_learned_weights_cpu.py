"""The learned TRSK weights on the host: the weights rebuilt from corrected
kite fractions keep TRSK's structure (calc_trisk_weights restated, the
Coriolis term does no work for any correction that sums to zero per cell),
the least-squares targets lower TRSK's reconstruction error, and the
network inputs have the documented form."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import fields, learned, learned_weights as lw


def test_weights_of_plain_kites_equal_the_reference_restatement(grid_at):
    g = grid_at(4)
    w = lw.trsk_weights(g.nnb, g.hx_hxtr_area.reshape(g.nv, 6))
    assert np.array_equal(w, oracle.trsk_weights(g))
    assert np.array_equal(w, g.hx_trskw.reshape(g.nv, 6, 6))


@pytest.mark.parametrize("level", [3, 5])
def test_any_sum_zero_correction_keeps_the_coriolis_term_work_free(grid_at, level):
    """sum_e l_e d_e F_e Q_perp_e = 0 (swm.f90:628-718) holds for the weights
    of any kite fractions that sum to one: the learned scheme conserves
    energy as TRSK does."""
    g = grid_at(level)
    rng = np.random.default_rng(level)
    x, cell, slot = lw.kite_inputs(g)
    R, w = lw.apply_outputs(g, rng.normal(0.0, 1.0, cell.size), cell, slot)
    n = g.nnb
    assert np.allclose(R.sum(axis=1), 1.0, atol=1e-14)
    assert np.abs(R - g.hx_hxtr_area.reshape(g.nv, 6)).max() > 0.05
    g2 = lw.with_weights(g, R, w)
    h, u = fields.balanced_state(g, lmax=10, seed=3)
    o = oracle.Oracle(g2, 2)
    o.tendency(h, u)
    work = o.field("uh") * o.field("uhq_perp") * g.ed_leng * g.edhx_leng * 0.5
    assert abs(np.sum(work)) <= 1e-13 * np.sum(np.abs(work))
    del n


def test_least_squares_targets_lower_the_reconstruction_error(grid_at):
    g = grid_at(4)
    dR = lw.lsq_targets(g, range(8), lmax=6, iters=1500)
    assert np.allclose(dR.sum(axis=1), 0.0, atol=1e-14)
    R = g.hx_hxtr_area.reshape(g.nv, 6) + dR
    g2 = lw.with_weights(g, R, lw.trsk_weights(g.nnb, R))
    for seed in (500, 501):
        u, ut = learned.velocity_sample(g, lmax=6, seed=seed)
        e0, e1 = lw.reconstruction_error(g, u, ut), lw.reconstruction_error(g2, u, ut)
        assert e1 < e0 / 2.0, (seed, e0, e1)


def test_kite_inputs_form(grid_at):
    g = grid_at(3)
    x, cell, slot = lw.kite_inputs(g)
    assert x.shape == (int(g.nnb.sum()), 24) and x.dtype == np.float32
    assert np.all(x[:, 14:] == 0.0)
    assert np.all(slot < g.nnb[cell])
    assert int(np.sum(x[:, 6])) == 12 * 5   # the pentagons' kites
    # slot-major order: slots never decrease
    assert np.all(np.diff(slot) >= 0)
    assert np.abs(x).max() < 20.0
