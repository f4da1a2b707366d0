"""TEST INFRASTRUCTURE ONLY: numpy FP64 reference of the closure MLP (the
checker for the CUDA training kernels' forward pass and gradients).

14-64-64-64-64-13, SiLU hidden activations, linear output, loss = mean of the
squared errors over samples and outputs; parameters per layer W [out][in]
row-major then b, as the library stores them."""
from __future__ import annotations

import numpy as np

DIMS = [14, 64, 64, 64, 64, 13]


def unpack(params: np.ndarray):
    layers, o = [], 0
    for i in range(len(DIMS) - 1):
        n_in, n_out = DIMS[i], DIMS[i + 1]
        W = params[o:o + n_out * n_in].reshape(n_out, n_in); o += n_out * n_in
        b = params[o:o + n_out]; o += n_out
        layers.append((W, b))
    assert o == params.size
    return layers


def num_params() -> int:
    return sum(DIMS[i + 1] * DIMS[i] + DIMS[i + 1] for i in range(len(DIMS) - 1))


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, X):
    a = X
    for W, b in unpack(params)[:-1]:
        a = silu(a @ W.T + b)
    W, b = unpack(params)[-1]
    return a @ W.T + b


def loss_and_grad(params, X, Y):
    layers = unpack(params)
    acts, zs = [X], []
    a = X
    for W, b in layers[:-1]:
        z = a @ W.T + b
        zs.append(z)
        a = silu(z)
        acts.append(a)
    W, b = layers[-1]
    y = a @ W.T + b
    n = X.shape[0] * Y.shape[1]
    r = y - Y
    loss = (r * r).sum() / n
    delta = 2.0 * r / n
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        W, b = layers[li]
        gW = delta.T @ acts[li]
        gb = delta.sum(axis=0)
        grads.append((gW, gb))
        if li > 0:
            delta = (delta @ W) * dsilu(zs[li - 1])
    grads.reverse()
    return loss, np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def forward_physical(params, norm, X):
    """Network in physical units: inputs normalised by (mean, std), outputs
    de-normalised; `norm` = input mean (14), input std (14), output mean (13),
    output std (13).  Returns (Y, Jacobian of the first six outputs with respect
    to the first six inputs, n x 6 x 6)."""
    nin, nout = DIMS[0], DIMS[-1]
    im, is_ = norm[:nin], norm[nin:2 * nin]
    om, os_ = norm[2 * nin:2 * nin + nout], norm[2 * nin + nout:]
    a = (X - im) / is_
    layers = unpack(params)
    # forward-mode tangents of the six strain inputs
    t = np.zeros((X.shape[0], 6, nin))
    for j in range(6):
        t[:, j, j] = 1.0 / is_[j]
    for W, b in layers[:-1]:
        z = a @ W.T + b
        t = dsilu(z)[:, None, :] * (t @ W.T)
        a = silu(z)
    W, b = layers[-1]
    y = (a @ W.T + b) * os_ + om
    J = (t @ W.T)[:, :, :6] * os_[:6]          # [n, j, o]
    return y, np.transpose(J, (0, 2, 1))       # [n, o, j]
