"""The numpy restatement of the band-tail MLP (oracle/mlp_ref.py): its BF16
rounding and its analytic gradient, by finite differences (CPU only)."""
from __future__ import annotations

import numpy as np

from oracle import mlp_ref


def test_bf16_round_to_nearest_even():
    # BF16 keeps 7 explicit mantissa bits: the unit at 1 is 2^-7
    x = np.array([1.0, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, 1 + 1.5 * 2.0 ** -8, 3.14159265, 0.0], dtype=np.float32)
    r = mlp_ref.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # halfway, ties to the even mantissa (0)
    assert r[2] == 1 + 2.0 ** -6            # halfway between mantissas 1 and 2: to 2
    assert r[3] == 1 + 2.0 ** -7            # above halfway: up
    assert r[4] == np.float32(3.140625)
    assert r[5] == 0.0
    y = np.random.default_rng(3).standard_normal(1000).astype(np.float32)
    assert np.all(np.abs(mlp_ref.bf16_round(y) - y) <= np.abs(y) * 2.0 ** -8)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    nin, nhid, nout, n = 5, 16, 3, 12
    npar = nhid * nin + nhid + nhid * nhid + nhid + nout * nhid + nout
    p = rng.standard_normal(npar) * 0.3
    x = rng.standard_normal((n, nin))
    t = rng.standard_normal((n, nout))
    L, g = mlp_ref.loss_and_grad(p, x, t, nin, nhid, nout, bf16=False)
    # float32 parameters: central differences in float64 on the float32 grid are
    # not smooth enough, so check in float64 by calling the float64 path directly
    def loss(pp):
        W1, b1, W2, b2, W3, b3 = mlp_ref.unpack(pp, nin, nhid, nout)
        H1 = np.maximum(x @ W1.T + b1, 0)
        H2 = np.maximum(H1 @ W2.T + b2, 0)
        Y = H2 @ W3.T + b3
        return np.mean((Y - t) ** 2)
    p64 = np.asarray(p, dtype=np.float32).astype(np.float64)
    h = 1e-6
    idx = rng.choice(npar, 40, replace=False)
    num = np.array([(loss(p64 + h * np.eye(npar)[i]) - loss(p64 - h * np.eye(npar)[i])) / (2 * h) for i in idx])
    assert np.allclose(g[idx], num, rtol=1e-5, atol=1e-8)
    assert abs(L - loss(p64)) < 1e-12
