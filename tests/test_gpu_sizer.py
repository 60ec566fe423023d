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


@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("dims,n", [((12, 32, 32, 1), 200), ((1, 32, 32, 1), 5000), ((12, 64, 64, 1), 3000),
                                    ((12, 16, 8, 1), 200)])
def test_gradients_match_oracle(gpu, fused, dims, n):
    """fp32 kernels against float64 backpropagation: |g - g_ref| <= 1e-3 * max|g_ref| + 1e-6, for
    the fused trainer (one cooperative launch, gradients summed per CTA then over CTAs) and the
    layer-by-layer kernels ((12, 16, 8, 1) is not a fused shape: layer by layer either way)."""
    try:
        omg.lib().omg_debug_set_fused_training(fused)
        m = sz.SizingModel(dims, seed=4)
        rng = np.random.default_rng(2)
        X = rng.random((n, dims[0])).astype(np.float32)
        T = rng.random(n).astype(np.float32)
        g, loss = m.gradients(X, T)
        ref_loss, ref_g = mlp_ref.loss_and_grad(m.get_params().astype(np.float64), m.dims, X.astype(np.float64),
                                                T.astype(np.float64))
        assert abs(loss - ref_loss) <= 1e-4 * max(ref_loss, 1e-6)
        np.testing.assert_allclose(g, ref_g, rtol=0, atol=1e-3 * np.abs(ref_g).max() + 1e-6)
        m.close()
    finally:
        omg.lib().omg_debug_set_fused_training(1)


def test_fused_and_layer_by_layer_training_agree(gpu):
    """The same model trained fused and layer by layer: Adam steps of at most lr per weight, so
    their weights stay within a few steps of each other and their losses agree."""
    rng = np.random.default_rng(8)
    X = rng.random((2048, 12)).astype(np.float32)
    T = (0.5 * X[:, 0] + 0.25 * np.sin(3 * X[:, 1]) + 0.1 * X[:, 2] * X[:, 3]).astype(np.float32)
    out = {}
    try:
        for fused in (1, 0):
            omg.lib().omg_debug_set_fused_training(fused)
            m = sz.SizingModel((12, 64, 64, 1), seed=9)
            m.train(X, T, epochs=300, lr=1e-3)
            out[fused] = (m.get_params(), float(np.mean((m.predict(X) - T) ** 2)))
            m.close()
    finally:
        omg.lib().omg_debug_set_fused_training(1)
    (p1, l1), (p0, l0) = out[1], out[0]
    assert np.median(np.abs(p1 - p0)) < 1e-3 and np.abs(p1 - p0).max() < 0.3
    assert abs(l1 - l0) <= 0.2 * max(l0, 1e-4), (l1, l0)


def test_learned_splits_train_in_milliseconds(gpu):
    """The CDF network of the learned range partitioner (1 -> 32 -> 32 -> 1, 16,384 points, 2,000
    Adam epochs) trains in one fused launch; the splits cut a skewed sample into near-equal ranges."""
    import time
    rng = np.random.default_rng(10)
    sample = (rng.zipf(1.3, 1 << 16) % (1 << 30)).astype(np.int64)
    omg.learn_splits(sample, bits=8, epochs=10)  # warm-up: module load, allocations
    t0 = time.perf_counter()
    splits = omg.learn_splits(sample, bits=8, epochs=2000)
    ms = (time.perf_counter() - t0) * 1e3
    print(f"learned 255 splits from {len(sample)} keys in {ms:.1f} ms")
    assert ms < 500, ms
    assert np.all(np.diff(splits) >= 0)


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
