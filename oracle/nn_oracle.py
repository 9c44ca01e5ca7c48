"""CPU oracle of the learned initial guess's network (test infrastructure only).

The reference has no learned component; this file is the checker of the
library's network kernels (midas_gb300/csrc/nn.cu): a float64 numpy
restatement of the same computation -- four 3x3x3 zero-padded convolutions,
16 -> 32 -> 32 -> 32 -> 8 channels (the last two output channels zero), ReLU
between them, the prediction E = E_inc + mask * out[:, :6] and the loss

    L = mean_b  sum(mask |E_pred - target|^2) / sum(mask |target|^2)

with its gradient for every parameter by backpropagation.  The forward pass
rounds where the GPU keeps fp16 values (the network inputs, the weights, the
post-ReLU activations), so the two agree up to the GPU's FP32 accumulation and
its fp16 gradient operands.  The restatement itself is pinned by finite
differences (tests/test_oracle_nn.py).

Layout (as the library's): voxels x fastest, then y, then z; arrays
[batch][grid^3][channels]; weights [cout][27 taps (dz, dy, dx = -1..1, dx
fastest)][cin], biases [cout]; parameters concatenated layer by layer.
"""
from __future__ import annotations

import numpy as np

CI = (16, 32, 32, 32)
CO = (32, 32, 32, 8)
NOUT = 6


def param_shapes():
    return [((CO[l], 27, CI[l]), (CO[l],)) for l in range(4)]


def param_count() -> int:
    return sum(co * 27 * ci + co for ci, co in zip(CI, CO))


def unpack(theta):
    out, off = [], 0
    for ws, bs in param_shapes():
        nw = int(np.prod(ws))
        out.append((theta[off:off + nw].reshape(ws), theta[off + nw:off + nw + bs[0]]))
        off += nw + bs[0]
    return out


def _f16(x):
    return np.asarray(x, np.float64).astype(np.float16).astype(np.float64)


def _shifted(X, G, o):
    """X [B, G, G, G, C] (z, y, x) -> its neighbour at tap o, zero outside the grid."""
    dz, dy, dx = o // 9 - 1, (o // 3) % 3 - 1, o % 3 - 1
    Y = np.zeros_like(X)
    zs, ys, xs = (slice(max(0, -d), G - max(0, d)) for d in (dz, dy, dx))
    zd, yd, xd = (slice(max(0, d), G - max(0, -d)) for d in (dz, dy, dx))
    Y[:, zs, ys, xs, :] = X[:, zd, yd, xd, :]
    return Y


def conv(X, W, G):
    """X [B, V, C] -> [B, V, Cout]: sum over the 27 taps and the input channels."""
    B, V, C = X.shape
    X5 = X.reshape(B, G, G, G, C)
    out = np.zeros((B, G, G, G, W.shape[0]))
    for o in range(27):
        out += _shifted(X5, G, o) @ W[:, o, :].T
    return out.reshape(B, V, W.shape[0])


def conv_t(dZ, W, G):
    """The adjoint of conv: dX[u] = sum_o dZ[u - o] W[:, o, :]."""
    B, V, Co = dZ.shape
    D5 = dZ.reshape(B, G, G, G, Co)
    out = np.zeros((B, G, G, G, W.shape[2]))
    for o in range(27):
        out += _shifted(D5, G, 26 - o) @ W[:, o, :]
    return out.reshape(B, V, W.shape[2])


def conv_wgrad(dZ, X, G):
    """dW[co, o, ci] = sum_v dZ[v, co] X[v + o, ci]."""
    B, V, C = X.shape
    X5 = X.reshape(B, G, G, G, C)
    dW = np.zeros((dZ.shape[2], 27, C))
    for o in range(27):
        S = _shifted(X5, G, o).reshape(B * V, C)
        dW[:, o, :] = dZ.reshape(B * V, -1).T @ S
    return dW


def loss_and_grads(theta, inputs, mask, target, G, fp16=True):
    """inputs [B, V, 16], mask [B, V], target [B, V, 6]; returns (loss, gradient of theta)."""
    r = _f16 if fp16 else (lambda a: np.asarray(a, np.float64))
    params = unpack(np.asarray(theta, np.float64))
    B = inputs.shape[0]
    X = [r(inputs)]
    Z = []
    for l, (W, b) in enumerate(params):
        z = conv(X[-1], r(W), G) + b
        Z.append(z)
        if l < 3:
            X.append(r(np.maximum(z, 0.0)))
    out = Z[3][:, :, :NOUT]
    einc = np.asarray(inputs, np.float64)[:, :, 2:8]
    m = np.asarray(mask, np.float64)[:, :, None]
    tgt = np.asarray(target, np.float64)
    d = (einc + out - tgt) * m
    den = np.array([max(float(np.sum(m[b] * tgt[b] ** 2)), 1e-300) for b in range(B)])
    loss = float(np.sum(np.sum(d ** 2, axis=(1, 2)) / den) / B)
    dZ = np.zeros_like(Z[3])
    dZ[:, :, :NOUT] = 2.0 * d / (den[:, None, None] * B)
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, _ = params[l]
        grads[l] = (conv_wgrad(dZ, X[l], G), dZ.sum(axis=(0, 1)))
        if l > 0:
            dZ = conv_t(dZ, r(W), G) * (Z[l - 1] > 0)
    flat = np.concatenate([np.concatenate([g.ravel(), b]) for g, b in grads])
    return loss, flat
