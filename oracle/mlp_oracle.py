"""FP64 numpy restatement of the warm-start network (test infrastructure only).

Only ``tests/`` import this module, as the checker of the CUDA training and
inference kernels of ``cm_gb300/csrc/fe_mlp.cu``.  The network has no
counterpart in the reference (OpenCMISS-Iron starts Newton from the current
field, solver_routines.f90:17812); what is restated here is the textbook
multilayer perceptron with tanh hidden layers, a linear output layer, mean
squared error and Adam (Kingma & Ba, 2015), with the conventions of the
kernels: W_l is [out][in] row-major, h_{l+1} = act(h_l W_l^T + b_l).
"""
from __future__ import annotations

import numpy as np


def forward(params, x):
    """params: list of (W, b); returns the list of layer outputs h_0 .. h_L."""
    hs = [np.asarray(x, dtype=np.float64)]
    for l, (W, b) in enumerate(params):
        z = hs[-1] @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        hs.append(np.tanh(z) if l + 1 < len(params) else z)
    return hs


def mse(pred, target):
    d = pred - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def backward(params, hs, dy):
    """Gradients (dW, db) of every layer for the output gradient dy."""
    grads = [None] * len(params)
    dh = dy
    for l in range(len(params) - 1, -1, -1):
        W = np.asarray(params[l][0], np.float64)
        dz = dh if l + 1 == len(params) else dh * (1.0 - hs[l + 1] ** 2)
        grads[l] = (dz.T @ hs[l], dz.sum(axis=0))
        dh = dz @ W
    return grads


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
