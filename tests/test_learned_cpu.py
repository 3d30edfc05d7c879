"""Learned-correction inputs and the CPU oracle of the network (no GPU)."""
import numpy as np
import pytest

import oracle
from imodel_gb300 import learned, swm
from oracle import mlp_oracle as mo


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.001953125, -2.5e-3, 3.0e38], dtype=np.float32)
    b = mo.bf16(x)
    # 1 + 2^-8 lies exactly between two bf16 values: ties to even -> 1.0
    assert b[1] == np.float32(1.0)
    assert b[2] == np.float32(1.0078125)
    assert np.all(np.abs(b - x) <= np.abs(x) * 2.0 ** -8)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mo.init_params(1)
    x = mo.bf16(rng.normal(size=(64, 24)).astype(np.float32))
    t = rng.normal(size=64).astype(np.float32)
    # compare only parameters that do not feed a BF16 rounding point, where
    # finite differences are smooth: b1, b2, w3, b3
    _, g = mo.loss_and_grad(p, x, t)
    P = mo.unpack(np.arange(mo.NPARAM))
    for name in ("b2", "w3", "b3"):
        for k in np.asarray(P[name], dtype=np.int64).ravel()[:6]:
            e = 1e-3
            pp, pm = p.copy(), p.copy()
            pp[k] += e
            pm[k] -= e
            fd = (mo.loss_and_grad(pp, x, t)[0] - mo.loss_and_grad(pm, x, t)[0]) / (2 * e)
            assert abs(fd - g[k]) <= 2e-3 * max(1.0, abs(g[k])), (name, k, fd, g[k])


def test_stencil_matches_trsk_tangent(grid_at):
    """The feature stencil reproduces vecrecon_trsk_tg exactly."""
    g = grid_at(4)
    _, u = swm.initialize_fields_tc2(g)
    u = u + np.random.default_rng(2).normal(0, 1.0, g.ne)
    a = learned.trsk_tangent_np(g, u)
    b = oracle.Oracle(g, 2).trsk_tangent(u)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)


def test_features_shape_and_scale(grid_at):
    g = grid_at(3)
    u, ut = learned.velocity_sample(g, lmax=12, seed=3)
    x, s = learned.features(g, u)
    assert x.shape == (g.ne, 24)
    # velocity inputs have unit RMS per edge
    np.testing.assert_allclose(np.mean(x[:, :10] ** 2, axis=1), 1.0, rtol=1e-12)
    # pentagon-adjacent edges have one zero velocity slot and one zero weight
    n_pad = np.sum(x[:, 10 + 4:] == 0.0, axis=1)
    assert set(np.unique(n_pad)) <= {0, 1, 2}


@pytest.mark.parametrize("level", [4, 6])
def test_velocity_sample_is_consistent(grid_at, level):
    """The exact tangential component of the sampled field is what TRSK
    approximates: the reconstruction error is a few percent, not O(1)."""
    g = grid_at(level)
    u, ut = learned.velocity_sample(g, lmax=16, seed=5)
    utg = learned.trsk_tangent_np(g, u)
    rel = np.sqrt(np.mean((utg - ut) ** 2) / np.mean(ut ** 2))
    assert rel < 0.1
