"""Laplacian diffusion and hyperdiffusion of the momentum in the oracle
(diffusion_ed / hyperdiffusion_ed, swm_operators.f90:855-975, constant
coefficients).  The operator is grad(K div u) - grad_tg(K zeta): the Hodge
vector Laplacian, which takes energy out of any flow.  Case 2's solid-body
rotation has no divergence, so only the vorticity term (and the sign of the
tangential gradient across each edge) acts there."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import fields, swm


def _work(g, d, u):
    """sum_e (l d / 2) u_e d_e: the rate of change of kinetic energy due to
    the extra momentum tendency d (up to the depth factor)."""
    return float(np.sum(0.5 * g.ed_leng * g.edhx_leng * u * d))


@pytest.mark.parametrize("level", [3, 4])
def test_diffusion_takes_energy_out(grid_at, level):
    g = grid_at(level)
    oracle.build()
    for h, u in (swm.initialize_fields_tc2(g), fields.balanced_state(g, lmax=12, seed=4)):
        _, m0 = oracle.Oracle(g, 2).tendency(h, u)
        _, m2 = oracle.Oracle(g, 2, k2=1.0e5).tendency(h, u)
        _, m4 = oracle.Oracle(g, 2, k4=1.0e15).tendency(h, u)
        lap, hyp = m2 - m0, m4 - m0
        assert np.abs(lap).max() > 0 and np.abs(hyp).max() > 0
        assert _work(g, lap, u) < 0
        assert _work(g, hyp, u) < 0


def test_diffusion_is_linear_in_the_coefficient(grid_at):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=5)
    _, m0 = oracle.Oracle(g, 2).tendency(h, u)
    _, m1 = oracle.Oracle(g, 2, k2=1.0e5).tendency(h, u)
    _, m2 = oracle.Oracle(g, 2, k2=2.0e5).tendency(h, u)
    np.testing.assert_allclose(m2 - m0, 2.0 * (m1 - m0), rtol=1e-6,
                               atol=1e-9 * np.abs(m1 - m0).max())


def test_negative_coefficient_refused(grid_at):
    with pytest.raises(ValueError):
        oracle.Oracle(grid_at(2), 2, k2=-1.0)
