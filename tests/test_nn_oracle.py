"""The learned warm start's CPU oracle: analytic gradients against central
finite differences in float64 (CPU only)."""
import numpy as np
import pytest

from oracle import nn_np as N


def _sample(H=16, W=8, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros((H, W, N.IN_CH))
    x[..., :N.FEATURES] = rng.standard_normal((H, W, N.FEATURES))
    target = rng.standard_normal((H, W))
    return x, target


def test_param_count():
    assert N.num_params() == sum(9 * a * b + b for _, a, b, _ in N.LAYERS)
    assert 600_000 < N.num_params() < 800_000


def test_backward_matches_finite_differences():
    x, target = _sample()
    flat = N.init_params(1)
    rng = np.random.default_rng(2)
    flat = flat + 0.01 * rng.standard_normal(flat.shape)     # break the zero biases
    y = N.forward(flat, x)
    loss, dy = N.mse_loss(y, target)
    g = N.backward(flat, x, dy)
    # probe parameters spread over every layer (weights and biases)
    offs, o = [], 0
    for _, cin, cout, _ in N.LAYERS:
        nw = 9 * cin * cout
        offs += [o + int(rng.integers(nw)), o + nw + int(rng.integers(cout))]
        o += nw + cout
    h = 1e-6
    for k in offs:
        e = np.zeros_like(flat)
        e[k] = h
        lp, _ = N.mse_loss(N.forward(flat + e, x), target)
        lm, _ = N.mse_loss(N.forward(flat - e, x), target)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)) + 1e-8, (k, fd, g[k])


def test_padded_channels_stay_inert():
    """Zero padding channels of the input and output never carry gradient to
    the live parameters' results."""
    x, target = _sample(seed=3)
    flat = N.init_params(4)
    y = N.forward(flat, x)
    assert np.all(y[..., 1:] == 0.0)


def test_adam_matches_closed_form_first_step():
    w = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -5.0, 0.0])
    w1, m, v = N.adam_step(w, g, np.zeros(3), np.zeros(3), 1, lr=0.1)
    # first step: m_hat = clip(g), v_hat = clip(g)^2  ->  w - lr * sign(g)
    assert np.allclose(w1, w - 0.1 * np.sign(np.clip(g, -1, 1)) * (np.abs(g) > 0), atol=1e-6)


def test_package_network_table_matches_oracle():
    """The host package (aerojax_gb300.nn) describes the same network as the
    oracle: layer table, parameter count and initialisation."""
    from aerojax_gb300 import nn as P
    assert [(a, b, int(r)) for a, b, r in P.LAYERS] == [(a, b, int(r)) for _, a, b, r in N.LAYERS]
    flat = P.init_params(3)
    assert flat.size == N.num_params()
    assert np.allclose(flat, N.init_params(3).astype(np.float32))
