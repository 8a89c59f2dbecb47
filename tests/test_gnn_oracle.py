"""The CPU restatement of the learned preconditioner (oracle/gnn_oracle.py)
checked against itself: analytic gradient vs central finite differences in
FP64, the BF16 rounding helper, and the chain matrix at gamma = 1 / alpha = 0
reproducing the block-tridiagonal part of S."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import gnn_oracle as G  # noqa: E402


def test_bf16_rounding():
    # BF16 keeps 8 significant bits: the spacing above 1.0 is 2^-7.
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, 1.0 + 3 * 2.0 ** -9, -2.5, 0.0, 3.0e38])
    r = G.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                        # halfway, ties to the even neighbour 1.0
    assert r[2] == 1.0 + 2.0 ** -6            # halfway between 1 + 2^-7 (odd) and 1 + 2^-6 (even)
    assert r[3] == 1.0                        # below halfway
    assert r[4] == 1.0 + 2.0 ** -7            # above halfway
    assert r[5] == -2.5 and r[6] == 0.0
    assert np.isfinite(r[7])


def test_chain_matrix_identity_coefficients():
    cp = G.random_chain_problem(n=9, seed=3)
    coef = np.zeros((cp.n, 3)); coef[:, 0] = coef[:, 1] = 1.0
    T, _ = cp.dense_T(coef)
    S = cp.dense_S()
    tri = np.zeros_like(S)
    for k in range(cp.n):
        for j in (k - 1, k, k + 1):
            if 0 <= j < cp.n:
                tri[15 * k:15 * k + 15, 15 * j:15 * j + 15] = S[15 * k:15 * k + 15, 15 * j:15 * j + 15]
    np.testing.assert_allclose(T, tri, atol=1e-14)


def test_gradient_matches_finite_differences():
    cp = G.random_chain_problem(n=10, seed=1)
    rng = np.random.default_rng(7)
    L, total = G.layout()
    params = rng.normal(size=total) * 0.2
    o, _ = L["bh"]
    params[o:o + 3] = [0.5, -0.3, -1.0]
    probes = rng.normal(size=(2, 15 * cp.n))
    loss, grad, _, _ = G.loss_and_grad(cp, params, probes, use_bf16=False)
    assert loss > 0
    idx = []
    for name, (off, shp) in L.items():
        size = int(np.prod(shp))
        idx += list(off + rng.choice(size, min(3, size), replace=False))
    h = 1e-6
    for i in idx:
        pp = params.copy(); pp[i] += h
        pm = params.copy(); pm[i] -= h
        lp = G.loss_and_grad(cp, pp, probes, use_bf16=False)[0]
        lm = G.loss_and_grad(cp, pm, probes, use_bf16=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-4 * abs(fd), (i, fd, grad[i])
