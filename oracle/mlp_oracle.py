"""FP64 CPU oracle of the learned cost model's MLP (test infrastructure only).

Same parameter layout as the library's ``pq_mlp``: one flat vector ordered
W1 b1 W2 b2 ... with W_l row-major [in x out]; ReLU after every hidden layer;
loss = mean((y_pred - y)^2).
"""
from __future__ import annotations

import numpy as np


def layer_shapes(n_in, hidden, layers):
    shapes = []
    w = n_in
    for _ in range(layers):
        shapes.append((w, hidden))
        w = hidden
    shapes.append((w, 1))
    return shapes


def unpack(params, n_in, hidden, layers):
    out, pos = [], 0
    for din, dout in layer_shapes(n_in, hidden, layers):
        W = params[pos:pos + din * dout].reshape(din, dout)
        pos += din * dout
        b = params[pos:pos + dout]
        pos += dout
        out.append((W, b))
    assert pos == len(params)
    return out


def forward(params, X, n_in, hidden, layers):
    acts = [np.asarray(X, np.float64)]
    Ls = unpack(np.asarray(params, np.float64), n_in, hidden, layers)
    for i, (W, b) in enumerate(Ls):
        z = acts[-1] @ W + b
        if i + 1 < len(Ls):
            z = np.maximum(z, 0.0)
        acts.append(z)
    return acts


def loss_and_grad(params, X, y, n_in, hidden, layers):
    """MSE loss and its gradient (flat, same layout as the parameters)."""
    acts = forward(params, X, n_in, hidden, layers)
    Ls = unpack(np.asarray(params, np.float64), n_in, hidden, layers)
    n = len(y)
    pred = acts[-1][:, 0]
    d = pred - np.asarray(y, np.float64)
    loss = float(np.mean(d * d))
    dz = (2.0 * d / n)[:, None]
    grads = []
    for i in range(len(Ls) - 1, -1, -1):
        W, _ = Ls[i]
        gW = acts[i].T @ dz
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if i > 0:
            dz = (dz @ W.T) * (acts[i] > 0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.reshape(-1), gb]) for gW, gb in grads])
    return loss, flat
