"""Test infrastructure: a numpy restatement of the band-tail MLP's arithmetic.

The band-tail network has no counterpart in the reference (it is an extension
of the reference's full band sum, which stays its target and its error
measure), so this
module restates the library's own definition (respackdev_gb300/csrc/rp_mlp.cu)
in float64 numpy, to check the GPU forward pass, loss and gradients:

    H1 = relu(X W1^T + b1),  H2 = relu(H1 W2^T + b2),  Y = H2 W3^T + b3,
    L  = mean((Y - T)^2) over samples and outputs,

with the weights and biases rounded to BF16 (round to nearest even) before
use, as the GPU passes read them; the gradient with respect to a master
(FP32) parameter is the gradient with respect to its BF16 copy.  Only
tests/ import this module.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a: np.ndarray) -> np.ndarray:
    """FP32 values rounded to the nearest BF16 (ties to even), returned as float32."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, nin: int, nhid: int, nout: int):
    """Split a flat parameter vector in the library's order."""
    p = np.asarray(params)
    sizes = [nhid * nin, nhid, nhid * nhid, nhid, nout * nhid, nout]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(nhid, nin), b1, W2.reshape(nhid, nhid), b2, W3.reshape(nout, nhid), b3


def forward(params, x, nin, nhid, nout, bf16=True):
    """Y and the pre-activations (Z1, Z2) and activations (H1, H2), float64."""
    q = bf16_round(params) if bf16 else np.asarray(params, dtype=np.float32)
    W1, b1, W2, b2, W3, b3 = [v.astype(np.float64) for v in unpack(q, nin, nhid, nout)]
    X = np.asarray(x, dtype=np.float64)
    Z1 = X @ W1.T + b1
    H1 = np.maximum(Z1, 0.0)
    Z2 = H1 @ W2.T + b2
    H2 = np.maximum(Z2, 0.0)
    Y = H2 @ W3.T + b3
    return Y, (X, Z1, H1, Z2, H2)


def loss_and_grad(params, x, t, nin, nhid, nout, bf16=True):
    """Mean squared error and its gradient (flat, the library's order)."""
    q = bf16_round(params) if bf16 else np.asarray(params, dtype=np.float32)
    W1, b1, W2, b2, W3, b3 = [v.astype(np.float64) for v in unpack(q, nin, nhid, nout)]
    Y, (X, Z1, H1, Z2, H2) = forward(params, x, nin, nhid, nout, bf16)
    T = np.asarray(t, dtype=np.float64)
    n = Y.size
    D = Y - T
    L = float(np.sum(D * D) / n)
    dY = 2.0 * D / n
    gW3 = dY.T @ H2
    gb3 = dY.sum(0)
    dH2 = (dY @ W3) * (Z2 > 0)
    gW2 = dH2.T @ H1
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2) * (Z1 > 0)
    gW1 = dH1.T @ X
    gb1 = dH1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return L, g
