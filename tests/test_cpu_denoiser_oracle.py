"""The denoiser's CPU restatement (oracle/denoiser.py) pinned by finite differences:
its analytic gradient matches central differences of its own loss along random
directions, and its bf16 rounding matches IEEE round-to-nearest-even."""
import numpy as np

from oracle import denoiser as D


def test_gradient_matches_finite_differences():
    net = D.UNet([2, 3, 4], in_channels=3, seed=1)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 8, 8, 8, 3))
    t = rng.normal(size=(2, 8, 8, 8))
    loss, g, _ = net.gradient(x, t)
    assert loss > 0
    p0 = net.params.copy()
    for _ in range(4):
        u = rng.normal(size=net.n_params)
        eps = 1e-6
        net.params = p0 + eps * u
        lp = np.abs(net.forward(x)[0] - t).mean()
        net.params = p0 - eps * u
        lm = np.abs(net.forward(x)[0] - t).mean()
        net.params = p0
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ u) <= 1e-6 * max(1.0, abs(fd))


def test_single_level_network_and_adam():
    net = D.UNet([2], in_channels=2, seed=3)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, 4, 4, 4, 2))
    t = rng.normal(size=(1, 4, 4, 4))
    loss0, g, _ = net.gradient(x, t)
    m = np.zeros_like(g)
    v = np.zeros_like(g)
    for step in range(1, 30):
        loss, g, _ = net.gradient(x, t)
        D.adam_step(net.params, g, m, v, step, 1e-2)
    assert loss < loss0


def test_round_bf16():
    vals = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40], dtype=np.float32)
    r = D.round_bf16(vals)
    assert r[0] == 1.0
    assert r[1] == 1.0  # halfway between 1 and 1 + 2^-7: ties to even
    assert r[2] == 1.0078125
    assert r[3] == -2.5
    assert np.isfinite(r[4])
