"""Spark decimal AVG on the GPU against the oracle (AverageSparkDecimalAggregator,
average_spark_decimal_aggregator.h): a checked sum with sticky overflow over the non-NULL values,
then CalcAvg's rescale / divide / round half away from zero / rescale; single stage for decimal64
and decimal128 inputs (with overflowing groups), and partial -> final two-stage."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, run_agg

pytestmark = pytest.mark.gpu

L = omg.LongType()
AVG, SUM, CNT = omg.OMNI_AGGREGATION_TYPE_AVG, omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN
M64 = (1 << 64) - 1


def _dec128(vals):
    return np.array([[v & M64, (v >> 64) & M64] for v in vals], dtype=np.uint64)


def _data(case, n, groups, seed):
    rng = np.random.default_rng(seed)
    key = rng.integers(0, groups, n).astype(np.int64)
    nulls = (rng.random(n) < 0.05) | (key % 31 == 0)
    if case == "dec128":
        vals = [int(rng.integers(-10**18, 10**18)) * 10**int(rng.integers(0, 20)) for _ in range(n)]
        for i in range(n):
            if key[i] % 13 == 0:  # groups that overflow 38 digits (in some row order or at the end)
                vals[i] = (1 if i % 3 else -1) * 4 * 10**37
        return key, _dec128(vals), nulls, oracle.T_DEC128, omg.Decimal128Type(38, 4), omg.Decimal128Type(38, 8)
    if case == "dec64_small":
        vals = rng.integers(-10**6, 10**6, n).astype(np.int64)
        return key, vals, nulls, oracle.T_DEC64, omg.Decimal64Type(7, 2), omg.Decimal64Type(11, 6)
    vals = rng.integers(-10**17, 10**17, n).astype(np.int64)
    return key, vals, nulls, oracle.T_DEC64, omg.Decimal64Type(18, 2), omg.Decimal128Type(22, 6)


def _oracle(key, col, nulls, in_t, it, ot):
    out_t = oracle.T_DEC128 if ot.id == omg.OMNI_DECIMAL128 else oracle.T_DEC64
    return oracle.hashagg([key], [oracle.T_LONG], [None],
                          [dict(func=oracle.F_AVG, col=col, in_type=in_t, out_type=out_t, nulls=nulls,
                                in_prec=it.precision, in_scale=it.scale, out_scale=ot.scale)], overflow_as_null=True)


@pytest.mark.parametrize("case", ["dec64", "dec64_small", "dec128"])
@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL, omg.AGG_STRATEGY_PARTITIONED])
def test_single_stage_decimal_avg(gpu, case, strategy):
    key, col, nulls, in_t, it, ot = _data(case, 120_000, 2500, 3)
    cols, _ = run_agg([0], [L], [[1]], [[it]], [[ot]], [AVG], [key, col], [L, it], nulls=[None, nulls],
                      strategy=strategy, overflow_as_null=True, batch_sizes=(4096, 1500))
    assert_agg_equal(cols, _oracle(key, col, nulls, in_t, it, ot), 1)


def test_decimal_avg_overflow_raises_without_overflow_as_null(gpu):
    key = np.zeros(4, dtype=np.int64)
    t = omg.Decimal128Type(38, 0)
    col = _dec128([6 * 10**37] * 3 + [1])
    with pytest.raises(omg.OmgError):
        run_agg([0], [L], [[1]], [[t]], [[t]], [AVG], [key, col], [L, t])


def _columns(batches):
    parts = [omg.batch_to_numpy(b) for b in batches]
    for b in batches:
        omg.free_batch(b)
    return [(np.concatenate([p[c][0] for p in parts]), np.concatenate([p[c][1] for p in parts]))
            for c in range(len(parts[0]))]


def test_partial_then_final_decimal_avg(gpu):
    """Partial AVG emits (sum as decimal(p + 10, s), count); the final AVG over the partials of
    three operators equals the single-stage result."""
    key, col, nulls, in_t, it, ot = _data("dec64", 90_000, 1200, 7)
    part_t = omg.Decimal128Type(28, 2)
    part = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[it]], [[part_t, L]], [AVG], output_partials=[True])
    partials = []
    checks = []
    for s, e in ((0, 30_000), (30_000, 70_000), (70_000, 90_000)):
        op = part.create_operator()
        for b0 in range(s, e, 4096):
            b1 = min(e, b0 + 4096)
            op.add_input(omg.make_batch([L, it], [key[b0:b1], col[b0:b1]], [None, nulls[b0:b1]]))
        outs = op.drain()
        op.delete()
        cols = [omg.batch_to_numpy(b) for b in outs]
        checks.append((s, e, cols))
        partials += outs
    part.close()
    # Each partial: SUM (exact, rescaled by 0) and COUNT of its rows; an empty group gives 0, 0.
    for s, e, cl in checks:
        cols = [(np.concatenate([p[c][0] for p in cl]), np.concatenate([p[c][1] for p in cl])) for c in range(3)]
        ora = oracle.hashagg([key[s:e]], [oracle.T_LONG], [None],
                             [dict(func=oracle.F_SUM, col=col[s:e], in_type=oracle.T_DEC64, out_type=oracle.T_DEC128,
                                   nulls=nulls[s:e]),
                              dict(func=oracle.F_COUNT_COL, col=col[s:e], in_type=oracle.T_DEC64,
                                   out_type=oracle.T_LONG, nulls=nulls[s:e])])
        # the oracle's SUM is NULL for an empty group where the partial is 0: compare through COUNT
        empty = ora[2][1].astype(np.int64) == 0
        ora[2][0][empty] = 0
        ora[3][0][empty] = False
        assert_agg_equal(cols, ora, 1)
    fin = omg.HashAggregationOperatorFactory([0], [L], [[1, 2]], [[part_t, L]], [[ot]], [AVG], input_raws=[False],
                                             overflow_as_null=True)
    op = fin.create_operator()
    for b in partials:
        op.add_input(b)
    cols = _columns(op.drain())
    op.delete()
    fin.close()
    assert_agg_equal(cols, _oracle(key, col, nulls, in_t, it, ot), 1)
