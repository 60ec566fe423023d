"""Synthetic key distributions for training and evaluating the learned sizer.

A workload is N rows whose int64 keys are drawn from D distinct values, uniformly or Zipf(s)
by rank; rank r maps to a pseudo-random 64-bit key.  Sizes and parameters are drawn log-uniform
so that the training records cover the range an operator meets.
"""
from __future__ import annotations

import numpy as np


def _mix(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return (x ^ (x >> np.uint64(31))).view(np.int64)


def zipf_ranks(rng, n, domain, s):
    """n ranks in [0, domain) with P(r) proportional to (r + 1)^-s (inverse CDF)."""
    w = np.arange(1, domain + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(n)), domain - 1)


def keys(rng, n, domain, kind="uniform", s=1.1, salt=0):
    with np.errstate(over="ignore"):
        if kind == "uniform":
            r = rng.integers(0, domain, n)
        else:
            r = zipf_ranks(rng, n, domain, s)
        return _mix(r.astype(np.uint64) * np.uint64(0x100000001B3) + np.uint64(salt))


def random_workload(rng, n_min=1 << 18, n_max=1 << 20, d_max=1 << 22):
    """(keys, description) of one random workload of the training family."""
    n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
    domain = int(np.exp(rng.uniform(np.log(10), np.log(min(d_max, 8 * n)))))
    kind = "zipf" if rng.random() < 0.6 else "uniform"
    s = float(rng.uniform(0.6, 1.4))
    salt = int(rng.integers(0, 2**31))
    return keys(rng, n, domain, kind, s, salt), dict(n=n, domain=domain, kind=kind, s=s)
