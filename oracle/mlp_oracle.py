"""CPU oracle for the plan selector's perceptron (numpy, float64).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` may import this module, as the
checker of the CUDA forward / backward / Adam kernels of the selector.

The selector has no counterpart in the reference (heFFTe picks plan options
from fixed rules, ``include/heffte_plan_logic.h:131-176``); this module states
the network the CUDA code computes:

    h1 = relu(X W1 + b1), h2 = relu(h1 W2 + b2), y = h2 W3 + b3
    loss = mean over all B x out entries of (y - T)^2

with the parameter vector laid out as W1 [in x H], b1 [H], W2 [H x H], b2 [H],
W3 [H x out], b3 [out], row-major, and Adam with beta1 = 0.9, beta2 = 0.999,
eps = 1e-8 and bias correction.
"""
from __future__ import annotations

import numpy as np


def unpack(p, nin, nh, nout):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = []
    for shape in ((nin, nh), (nh,), (nh, nh), (nh,), (nh, nout), (nout,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    assert o == p.size
    return out


def forward(p, X, nin, nh, nout):
    W1, b1, W2, b2, W3, b3 = unpack(p, nin, nh, nout)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3, (X, h1, h2)


def loss_grad(p, X, T, nin, nh, nout):
    W1, b1, W2, b2, W3, b3 = unpack(p, nin, nh, nout)
    y, (X, h1, h2) = forward(p, X, nin, nh, nout)
    T = np.asarray(T, dtype=np.float64)
    n = y.size
    loss = float(np.sum((y - T) ** 2) / n)
    dy = 2.0 * (y - T) / n
    gW3, gb3 = h2.T @ dy, dy.sum(0)
    dh2 = (dy @ W3.T) * (h2 > 0)
    gW2, gb2 = h1.T @ dh2, dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    gW1, gb1 = X.T @ dh1, dh1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, g


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


def train(p, X, T, nin, nh, nout, steps, lr):
    p = np.asarray(p, dtype=np.float64).copy()
    m, v = np.zeros_like(p), np.zeros_like(p)
    loss = None
    for s in range(1, steps + 1):
        loss, g = loss_grad(p, X, T, nin, nh, nout)
        p, m, v = adam(p, g, m, v, s, lr)
    return p, loss
