"""ORACLE (test infrastructure only): FP64 numpy restatement of the cost
model's perceptron, to check the GPU kernels' forward pass and gradients.

Layout of the flat parameter vector (as gfft_mlp_get_params returns it): for
each layer l = 0..depth, W_l (out x in, row-major) then b_l (out); hidden
layers have ReLU, the last layer is linear with one output.  Loss: mean
squared error over the samples.
"""
from __future__ import annotations

import numpy as np


def unpack(p, nin, width, depth):
    layers = []
    off = 0
    for l in range(depth + 1):
        ni = nin if l == 0 else width
        no = 1 if l == depth else width
        W = p[off:off + ni * no].reshape(no, ni)
        off += ni * no
        b = p[off:off + no]
        off += no
        layers.append((W, b))
    assert off == len(p)
    return layers


def forward(p, X, nin, width, depth):
    layers = unpack(np.asarray(p, dtype=np.float64), nin, width, depth)
    a = np.asarray(X, dtype=np.float64)
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = z if l == depth else np.maximum(z, 0.0)
    return a[:, 0]


def gradients(p, X, y, nin, width, depth):
    """d/dp of mean((f(X) - y)^2), flat like p."""
    p = np.asarray(p, dtype=np.float64)
    layers = unpack(p, nin, width, depth)
    acts = [np.asarray(X, dtype=np.float64)]
    zs = []
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        zs.append(z)
        acts.append(z if l == depth else np.maximum(z, 0.0))
    n = len(y)
    delta = 2.0 * (acts[-1][:, 0] - np.asarray(y, dtype=np.float64))[:, None] / n
    grads = []
    for l in range(depth, -1, -1):
        W, b = layers[l]
        gW = delta.T @ acts[l]
        gb = delta.sum(0)
        grads.append((gW, gb))
        if l > 0:
            delta = (delta @ W) * (zs[l - 1] > 0)
    grads.reverse()
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
