"""Learned sizer on the GPU: the network's forward pass and gradients (CUDA kernels) against the
float64 restatement, training, and what the trained model gains over the plain sketch estimate
on workloads it was not trained on."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import omnioperator_gb300.sizer as sz
import omnioperator_gb300.sizer_data as sd
from oracle import mlp_ref

pytestmark = pytest.mark.gpu

L = omg.LongType()


def test_forward_matches_oracle(gpu):
    m = sz.SizingModel((12, 16, 8, 1), seed=3)
    rng = np.random.default_rng(1)
    X = rng.random((33, 12)).astype(np.float32)
    y = m.predict(X)
    ref, _ = mlp_ref.forward(m.get_params().astype(np.float64), m.dims, X.astype(np.float64))
    np.testing.assert_allclose(y, ref, rtol=2e-5, atol=2e-6)
    m.close()


def test_gradients_match_oracle(gpu):
    """fp32 kernels against float64 backpropagation: |g - g_ref| <= 1e-3 * max|g_ref| + 1e-6."""
    m = sz.SizingModel((12, 32, 32, 1), seed=4)
    rng = np.random.default_rng(2)
    X = rng.random((200, 12)).astype(np.float32)
    T = rng.random(200).astype(np.float32)
    g, loss = m.gradients(X, T)
    ref_loss, ref_g = mlp_ref.loss_and_grad(m.get_params().astype(np.float64), m.dims, X.astype(np.float64),
                                            T.astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-4 * max(ref_loss, 1e-6)
    np.testing.assert_allclose(g, ref_g, rtol=0, atol=1e-3 * np.abs(ref_g).max() + 1e-6)
    m.close()


def test_training_fits_a_smooth_function(gpu):
    rng = np.random.default_rng(5)
    X = rng.random((512, 12)).astype(np.float32)
    T = (0.5 * X[:, 0] + 0.25 * np.sin(3 * X[:, 1]) + 0.1 * X[:, 2] * X[:, 3]).astype(np.float32)
    m = sz.SizingModel((12, 32, 32, 1), seed=6)
    before = float(np.mean((m.predict(X) - T) ** 2))
    m.train(X, T, epochs=1500, lr=3e-3)
    after = float(np.mean((m.predict(X) - T) ** 2))
    assert after < 0.05 * before and after < 2e-3, (before, after)
    p = m.get_params()
    m2 = sz.SizingModel((12, 32, 32, 1), seed=99)
    m2.set_params(p)
    np.testing.assert_array_equal(m2.predict(X), m.predict(X))
    m.close()
    m2.close()


def _records(rng, count, **kw):
    """Sizing records logged by the plain operator (COUNT(*) by key) on random workloads."""
    fac = omg.HashAggregationOperatorFactory([0], [L], [[]], [[]], [[L]], [omg.OMNI_AGGREGATION_TYPE_COUNT_ALL])
    out = []
    for _ in range(count):
        keys, desc = sd.random_workload(rng, **kw)
        op = fac.create_operator()
        op.add_input(omg.make_batch([L], [keys]))
        omg.free_batches(op.drain())
        rec, groups = sz.record_from_operator(op)
        assert groups == len(np.unique(keys))
        out.append((rec, groups, desc))
        op.delete()
    fac.close()
    return out


def test_learned_estimate_beats_plain_estimate_on_held_out_workloads(gpu):
    rng = np.random.default_rng(7)
    train = _records(rng, 120)
    test = _records(rng, 40)
    X, T = sz.dataset([(r, g) for r, g, _ in train])
    m = sz.SizingModel(seed=8)
    m.train(X, T, epochs=3000, lr=3e-3)
    Xt, _ = sz.dataset([(r, g) for r, g, _ in test])
    pred = m.predict(Xt)
    learned = np.array([abs(np.log2(sz.estimate(r, y) / g)) for (r, g, _), y in zip(test, pred)])
    plain = np.array([abs(np.log2(r[20] / g)) for r, g, _ in test])  # r[20]: the plain estimate
    assert learned.mean() < 0.6 * plain.mean(), (learned.mean(), plain.mean())
    m.close()


def test_learned_sizing_avoids_resizes_and_stays_exact(gpu):
    """Attached to the factory, the model pre-sizes the table: on a skewed workload the plain
    estimate undersizes (and the exact path grows the table), the learned one does not; both
    give the same groups."""
    rng = np.random.default_rng(9)
    train = _records(rng, 120)
    X, T = sz.dataset([(r, g) for r, g, _ in train])
    m = sz.SizingModel(seed=10)
    m.train(X, T, epochs=3000, lr=3e-3)
    keys = sd.keys(np.random.default_rng(11), 1 << 20, 1 << 21, "zipf", 0.8, salt=5)
    groups = len(np.unique(keys))
    res = {}
    for learned in (False, True):
        fac = omg.HashAggregationOperatorFactory([0], [L], [[]], [[]], [[L]], [omg.OMNI_AGGREGATION_TYPE_COUNT_ALL])
        if learned:
            fac.set_sizer(m)
        op = fac.create_operator()
        op.add_input(omg.make_batch([L], [keys]))
        outs = op.drain()
        n = sum(omg.batch_row_count(b) for b in outs)
        omg.free_batches(outs)
        res[learned] = (n, op.counters()["resizes"], op.sizing_log())
        op.delete()
        fac.close()
    assert res[False][0] == res[True][0] == groups
    assert res[True][2]["learned"] and not res[False][2]["learned"]
    assert res[False][2]["estimate"] < 0.5 * groups  # the plain estimate undersizes this workload
    assert res[True][1] < res[False][1], res
    m.close()


@pytest.mark.parametrize("groups", [300, 40_000, 1_500_000])
def test_hll_sizing_estimates_the_group_count(gpu, groups):
    """The HyperLogLog sizing (every row's key, 2^14 registers) lands within 4% of the true group
    count on uniform and skewed keys (NULL keys counted as one group), and the result is exact."""
    rng = np.random.default_rng(groups)
    n = 1 << 22
    uniq = rng.integers(-2**62, 2**62, groups, dtype=np.int64)
    keys = uniq[np.minimum(rng.zipf(1.2, n) - 1, groups - 1)] if groups > 1000 else uniq[rng.integers(0, groups, n)]
    nulls = rng.random(n) < 0.001
    true = len(np.unique(keys[~nulls])) + 1
    fac = omg.HashAggregationOperatorFactory([0], [L], [[]], [[]], [[L]], [omg.OMNI_AGGREGATION_TYPE_COUNT_ALL])
    op = fac.create_operator()
    op.set_agg_sizing(omg.AGG_SIZING_HLL)
    op.add_input(omg.make_batch([L], [keys], [nulls]))
    outs = op.drain()
    got = sum(omg.batch_row_count(b) for b in outs)
    omg.free_batches(outs)
    est = op.sizing_log()["estimate"]
    op.delete()
    fac.close()
    assert got == true
    assert abs(est - true) <= 0.04 * true + 2, (est, true)
