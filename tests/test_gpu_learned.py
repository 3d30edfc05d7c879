"""Tensor-core network of the learned TRSK correction against the CPU oracle,
and what the trained network gains over plain TRSK."""
import numpy as np
import pytest

from imodel_gb300 import learned
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _rand_problem(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 24)).astype(np.float32)
    t = rng.normal(size=n).astype(np.float32)
    return learned.to_bf16_bits(x), mo.bf16(x), t


@pytest.mark.parametrize("n", [128, 1000])
def test_forward_matches_oracle(n):
    xb, x, _ = _rand_problem(n, 1)
    p = mo.init_params(3)
    p[mo.NPARAM - 1] = 0.25
    net = learned.Mlp(params=p)
    y = net.forward(xb)
    yr, _ = mo.forward(p, x)
    err = np.max(np.abs(y - yr)) / np.max(np.abs(yr))
    print(f"forward n={n}: max |y - y_oracle| / max |y| = {err:.2e}")
    # measured 2.1e-4 (n = 128) and 3.4e-4 (n = 1000) on a GB300: the
    # tensor cores and the oracle sum the FP32 products in different orders
    assert err < 3e-3
    assert np.mean(np.abs(y - yr)) < 1e-3 * np.mean(np.abs(yr)) + 1e-6


@pytest.mark.parametrize("batch,weighted", [(128, False), (300, True), (4096, True)])
def test_gradient_matches_oracle(batch, weighted):
    xb, x, t = _rand_problem(batch, 2)
    w = np.random.default_rng(8).uniform(0.1, 3.0, batch).astype(np.float32) if weighted else None
    p = mo.init_params(4)
    net = learned.Mlp(params=p)
    loss, g = net.grad(xb, t, w=w, batch=batch, seed=0)
    lr_, gr = mo.loss_and_grad(p, x, t, w)
    rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
    print(f"gradient batch={batch}: loss {loss:.6f} vs {lr_:.6f}, relative L2 {rel:.2e}")
    assert abs(loss - lr_) <= 1e-4 * lr_
    # measured 4.1e-4, 1.7e-4, 6.3e-5 for the three batches on a GB300
    assert rel < 4e-3
    P, G = mo.unpack(g), mo.unpack(gr)
    for name in ("W1", "b1", "W2", "b2", "w3", "b3"):
        r = np.linalg.norm(P[name] - G[name]) / (np.linalg.norm(G[name]) + 1e-30)
        print(f"  {name}: relative L2 {r:.2e}")
        assert r < 8e-3, (name, r)


def test_adam_training_reduces_loss():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(20000, 24)).astype(np.float32)
    w = rng.normal(size=24).astype(np.float32)
    t = np.tanh(x @ w / 5.0).astype(np.float32)
    net = learned.Mlp(params=mo.init_params(6))
    net.load_dataset(learned.to_bf16_bits(x), t)
    losses = net.train(200, batch=2048, lr=3e-3, seed=9)
    print(f"training: loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    assert losses[-1] < 0.2 * losses[0]


def test_learned_correction_beats_plain_trsk(grid_at):
    """Trained on seeded fields of one grid, the network lowers TRSK's
    tangential-reconstruction error on unseen fields of the same grid."""
    g = grid_at(5)
    # degree-12 fields resolved by ~14 cells per wavelength, as degree-48
    # fields are on level 7
    x, t, w = learned.training_set(g, seeds=range(24), lmax=12, mixtures=200)
    net = learned.Mlp(params=mo.init_params(0))
    net.load_dataset(x, t, w)
    losses = net.train(2000, batch=16384, lr=2e-3, seed=3)
    st = learned.stencil(g)
    gains = []
    for seed in (1000, 1001):
        u, ut = learned.velocity_sample(g, lmax=12, seed=seed)
        plain = learned.trsk_tangent_np(g, u, st)
        corr = learned.corrected_tangent(g, net, u, st)
        e0 = np.sqrt(np.mean((plain - ut) ** 2) / np.mean(ut ** 2))
        e1 = np.sqrt(np.mean((corr - ut) ** 2) / np.mean(ut ** 2))
        gains.append(e0 / e1)
        print(f"unseen field {seed}: TRSK rel L2 error {e0:.3e}, learned {e1:.3e}")
    print(f"training loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    assert min(gains) > 2.0
