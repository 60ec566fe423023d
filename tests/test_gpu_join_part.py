"""Partitioned inner join (hash and learned-range partitioning) against the oracle: the output
row multiset must equal the direct probe's and the oracle's, whatever the partition function."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
from helpers import expected_join_rows, join_rows_canonical

pytestmark = pytest.mark.gpu

L = omg.LongType()


def _zipf_ranks(rng, n, domain, s):
    w = np.arange(1, domain + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.minimum(np.searchsorted(cdf, rng.random(n)), domain - 1)


def _skewed(seed, nb, npb, s=1.1, nulls=0.01):
    """Build: 2*u for distinct u < 2^39, two int64 payloads; probe: 90% Zipf(s) over the build
    keys (through a random rank order), 10% odd keys (never match), `nulls` NULL."""
    rng = np.random.default_rng(seed)
    u = np.unique(rng.integers(0, 2**39, int(nb * 1.1)))[:nb]
    rng.shuffle(u)
    bkey = (2 * u).astype(np.int64)
    p1 = rng.integers(-2**62, 2**62, nb, dtype=np.int64)
    p2 = rng.integers(-2**62, 2**62, nb, dtype=np.int64)
    order = rng.permutation(nb)
    hit = bkey[order[_zipf_ranks(rng, npb, nb, s)]]
    miss = (rng.integers(0, 2**39, npb) * 2 + 1).astype(np.int64)
    pkey = np.where(rng.random(npb) < 0.9, hit, miss)
    pnull = rng.random(npb) < nulls
    return bkey, p1, p2, pkey, pnull


def _join(bkey, p1, p2, pkey, pnull, strategy=None, bits=8, splits=None, batch=None, device=True):
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L, L], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, L, L], [bkey, p1, p2]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [L, L], bf)
    op = pf.create_operator()
    if strategy is not None:
        op.set_join_strategy(strategy, bits, splits)
    op.set_no_more_input(False)
    n = len(pkey)
    step = n if batch is None else batch
    for s0 in range(0, n, step):
        b = omg.make_batch([L], [pkey[s0:s0 + step]], [pnull[s0:s0 + step]])
        if device:
            d = omg.batch_to_device(b)
            omg.free_batch(b)
            b = d
        op.add_input(b)
    op.no_more_input()
    outs = op.drain()
    per = [omg.batch_to_numpy(b) for b in outs]
    omg.free_batches(outs)
    ctr = op.counters()
    op.delete()
    pf.close()
    bop.delete()
    bf.close()
    cols = [(np.concatenate([p[c][0] for p in per]), np.concatenate([p[c][1] for p in per])) for c in range(3)] \
        if per else None
    return join_rows_canonical(cols), ctr


def _expected(bkey, p1, p2, pkey, pnull):
    return expected_join_rows([pkey], [pnull], [bkey, p1, p2], None, 0, 0, [0], [1, 2])


@pytest.mark.parametrize("s", [0.9, 1.3])
def test_hash_partitioned_matches_oracle(gpu, s):
    data = _skewed(1, 60_000, 500_000, s=s)
    got, _ = _join(*data, strategy=omg.JOIN_HASH_PARTITIONED, bits=10)
    assert got == _expected(*data)


def test_learned_range_partitioned_matches_oracle(gpu):
    data = _skewed(2, 50_000, 400_000, s=1.1)
    pkey, pnull = data[3], data[4]
    sample = pkey[~pnull][:: max(1, len(pkey) // 65536)]
    splits = omg.learn_splits(sample, bits=9, epochs=1000)
    assert len(splits) == 511 and np.all(np.diff(splits) >= 0)
    got, _ = _join(*data, strategy=omg.JOIN_RANGE_PARTITIONED, bits=9, splits=splits)
    assert got == _expected(*data)


def test_partitioned_from_many_host_batches(gpu):
    data = _skewed(3, 20_000, 150_000, s=1.0)
    got, _ = _join(*data, strategy=omg.JOIN_HASH_PARTITIONED, bits=6, batch=4096, device=False)
    assert got == _expected(*data)


def test_partitioned_equals_direct_probe(gpu):
    data = _skewed(4, 30_000, 200_000, s=1.2)
    direct, _ = _join(*data)
    part, _ = _join(*data, strategy=omg.JOIN_HASH_PARTITIONED, bits=12)
    assert direct == part


def test_duplicate_build_keys_keep_the_direct_probe(gpu):
    bkey, p1, p2, pkey, pnull = _skewed(5, 10_000, 50_000)
    bkey = np.concatenate([bkey, bkey[:100]])
    p1 = np.concatenate([p1, p1[:100] + 1])
    p2 = np.concatenate([p2, p2[:100]])
    got, _ = _join(bkey, p1, p2, pkey, pnull, strategy=omg.JOIN_HASH_PARTITIONED, bits=8)
    assert got == _expected(bkey, p1, p2, pkey, pnull)


def test_learned_splits_balance_a_skewed_sample(gpu):
    """Keys with a smooth but very uneven density over the key space (two narrow modes and empty
    space between them): equal-width ranges are badly unbalanced, the learned CDF's quantiles are
    not.  (The small network cannot resolve CDF steps much narrower than ~1e-3 of the key range,
    such as a few tight clusters; those keep whole clusters in one range.)"""
    rng = np.random.default_rng(6)
    modes = np.concatenate([rng.normal(0.3, 0.02, 32768), rng.normal(0.7, 0.03, 32768)])
    sample = (2.0**40 * modes).astype(np.int64)
    splits = omg.learn_splits(sample, bits=6, epochs=3000)
    counts = np.bincount(np.searchsorted(splits, sample, side="right"), minlength=64)
    width = np.linspace(sample.min(), sample.max(), 65)[1:-1].astype(np.int64)
    counts_w = np.bincount(np.searchsorted(width, sample, side="right"), minlength=64)
    assert counts.max() < 0.5 * counts_w.max()
    assert counts.max() <= 2.5 * len(sample) / 64


def test_fingerprint_is_order_independent_and_sensitive(gpu):
    rng = np.random.default_rng(7)
    a = rng.integers(-2**62, 2**62, 100_000, dtype=np.int64)
    b = rng.integers(-2**62, 2**62, 100_000, dtype=np.int64)
    m = rng.random(100_000) < 0.1
    perm = rng.permutation(100_000)
    x = [omg.make_batch([L, L], [a[:60_000], b[:60_000]], [m[:60_000], None]),
         omg.make_batch([L, L], [a[60_000:], b[60_000:]], [m[60_000:], None])]
    y = [omg.make_batch([L, L], [a[perm], b[perm]], [m[perm], None])]
    b2 = b.copy()
    b2[123] ^= 1
    z = [omg.make_batch([L, L], [a, b2], [m, None])]
    fx, fy, fz = omg.batches_fingerprint(x), omg.batches_fingerprint(y), omg.batches_fingerprint(z)
    assert fx == fy and fx[0] == 100_000
    assert fz[0] == fx[0] and fz[1:] != fx[1:]
    omg.free_batches(x + y + z)


@pytest.mark.parametrize("s", [0.9, 1.1, 1.3])
def test_quantile_choice_matches_learned_choice(gpu, s):
    """The strategy read off exact sample quantiles equals the one read off the learned splits
    (what the network adds to this decision: nothing), and both probes give the oracle's rows."""
    data = _skewed(8, 100_000, 400_000, s=s)
    pkey, pnull = data[3], data[4]
    sample = pkey[~pnull][:: max(1, len(pkey) // 65536)]
    learned = omg.learn_splits(sample, bits=10, epochs=1000)
    quantile = omg.quantile_splits(sample, bits=10)
    got_l, _ = _join(*data, strategy=omg.JOIN_LEARNED, bits=10, splits=learned)
    got_q, _ = _join(*data, strategy=omg.JOIN_QUANTILE, bits=10, splits=quantile)
    assert got_l == got_q == _expected(*data)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L], [0])
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1], [L], bf)
    op = pf.create_operator()
    op.set_join_strategy(omg.JOIN_LEARNED, 10, learned)
    chose_l = op.join_strategy()
    op.set_join_strategy(omg.JOIN_QUANTILE, 10, quantile)
    chose_q = op.join_strategy()
    op.delete()
    pf.close()
    bf.close()
    assert chose_l == chose_q
