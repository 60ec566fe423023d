"""Learned sizer, CPU side: the float64 network restatement used as the gradient oracle is
checked against central differences, and the feature / target / estimate transforms of the
library (host code, no GPU) against a direct computation."""
import math

import numpy as np

import omnioperator_gb300.sizer as sz
from oracle import mlp_ref


def _record(N, n, special, d, f1, f2=0, f3=0, f47=0, f8=0, mx=1, heavy=0):
    return [N, n, special, d, f1, f2, f3, f47, f8, mx, heavy] + [0] * 6


def test_oracle_backprop_matches_central_differences():
    rng = np.random.default_rng(0)
    dims = (5, 7, 6, 1)
    n_params = sum(k * m + m for k, m in zip(dims[:-1], dims[1:]))
    p = rng.standard_normal(n_params) * 0.5
    X = rng.standard_normal((9, 5))
    T = rng.standard_normal(9)
    _, g = mlp_ref.loss_and_grad(p, dims, X, T)
    num = mlp_ref.numeric_grad(p, dims, X, T)
    np.testing.assert_allclose(g, num, rtol=1e-5, atol=1e-8)


def test_features_of_a_record():
    rec = _record(N=1 << 22, n=65536, special=10, d=10_000, f1=98, f2=300, f3=500, f47=4000, f8=5102, mx=40,
                  heavy=50_000)
    x = sz.features(rec)
    n = 65536 - 10
    gee = min(max(math.sqrt((1 << 22) / n) * 98 + (10_000 - 98), 10_000), 1 << 22)
    exp = [math.log2((1 << 22) + 1) / 32, math.log2(n + 1) / 32, math.log2(10_001) / 32, 98 / n, 300 / n, 500 / n,
           4000 / n, 5102 / n, 50_000 / n, math.log2(41) / 16, math.log2((1 << 22) / n) / 16,
           math.log2(gee / 10_000) / 16]
    np.testing.assert_allclose(x, np.array(exp, dtype=np.float32), rtol=1e-6)


def test_target_and_estimate_invert():
    rec = _record(N=1 << 24, n=65536, special=0, d=40_000, f1=30_000)
    for g in (40_000, 1_000_000, 15_000_000):
        y = sz.target(rec, g)
        assert abs(sz.estimate(rec, y) - g) <= max(2, g * 1e-5)
    # clamped to [d, N]
    assert sz.estimate(rec, -1.0) == 40_000
    assert sz.estimate(rec, 10.0) == 1 << 24
