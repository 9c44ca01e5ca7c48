"""The network oracle (oracle/nn_oracle.py) pinned by finite differences.

Without fp16 rounding, the oracle's backpropagated gradient must equal the
central-difference derivative of its own loss, entry by entry and along a
random direction.
"""
import numpy as np

from oracle import nn_oracle as N


def _case(G=4, B=2, seed=0):
    rng = np.random.default_rng(seed)
    V = G ** 3
    inputs = rng.standard_normal((B, V, 16)) * 0.5
    mask = (rng.random((B, V)) < 0.6).astype(float)
    inputs[:, :, 0:2] *= mask[:, :, None]
    target = rng.standard_normal((B, V, 6))
    theta = rng.standard_normal(N.param_count()) * 0.1
    off = sum(co * 27 * ci + co for ci, co in zip(N.CI[:3], N.CO[:3]))
    W3 = theta[off:off + 8 * 27 * 32].reshape(8, 27, 32)   # padded output rows are zero
    W3[6:] = 0
    theta[off + 8 * 27 * 32 + 6:off + 8 * 27 * 32 + 8] = 0
    return theta, inputs, mask, target, G


def test_gradient_matches_finite_differences():
    theta, inputs, mask, target, G = _case()
    loss, g = N.loss_and_grads(theta, inputs, mask, target, G, fp16=False)
    rng = np.random.default_rng(1)
    h = 1e-6
    for i in rng.choice(len(theta), size=40, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (N.loss_and_grads(tp, inputs, mask, target, G, fp16=False)[0] -
              N.loss_and_grads(tm, inputs, mask, target, G, fp16=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (i, fd, g[i])
    assert loss > 0


def test_directional_derivative_of_whole_gradient():
    theta, inputs, mask, target, G = _case(seed=3)
    _, g = N.loss_and_grads(theta, inputs, mask, target, G, fp16=False)
    d = np.random.default_rng(4).standard_normal(len(theta))
    h = 1e-6
    fd = (N.loss_and_grads(theta + h * d, inputs, mask, target, G, fp16=False)[0] -
          N.loss_and_grads(theta - h * d, inputs, mask, target, G, fp16=False)[0]) / (2 * h)
    assert abs(fd - g @ d) <= 1e-6 * abs(fd)
