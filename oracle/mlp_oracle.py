"""FP64 numpy restatement of the surrogate MLP (TEST INFRASTRUCTURE ONLY).

Forward: h_{l+1} = GELU(h_l W_l^T + b_l) for the hidden layers, y = h_L W_L^T + b_L, loss =
mean((y - t)^2).  Backward by the chain rule, with GELU'(x) = Phi(x) + x phi(x) (erf form).
Used to check the gradients of the hand-written CUDA kernels (elanfmt_gb300/surrogate.py);
self-checked against central finite differences in tests/test_surrogate_cpu.py.
"""
from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward(x, Ws, bs):
    """Returns (y, hs, pres): hs[l] is the input of layer l, pres[l] its pre-activation."""
    h = np.asarray(x, np.float64)
    hs, pres = [h], []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = h @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        pres.append(z)
        h = gelu(z) if l < len(Ws) - 1 else z
        hs.append(h)
    return h, hs, pres


def loss_and_grads(x, t, Ws, bs):
    y, hs, pres = forward(x, Ws, bs)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    dy = 2.0 * (y - t) / n
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        gW[l] = dy.T @ hs[l]
        gb[l] = dy.sum(axis=0)
        if l > 0:
            dh = dy @ np.asarray(Ws[l], np.float64)
            dy = dh * gelu_grad(pres[l - 1])
    return loss, gW, gb
