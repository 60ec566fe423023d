"""Two-stage Spark decimal SUM on the GPU against the oracle's restatement.

A partial stage emits (decimal sum, boolean isEmpty) per group: the sum NULL when it overflowed,
0 with isEmpty TRUE for a group without values (sum_spark_decimal_aggregator.h:165-241).  A
merging stage skips isEmpty rows, takes a NULL partial sum as an overflow and adds the other
partial sums with the checked, sticky addition in arrival order (AddDecimalUseRowIndex,
:14-66); its output is the final sum (NULL, or an error, on overflow) or again a partial pair.
Partial sums near 10^38 make some groups overflow, some only on a prefix of their rows (an
order-dependent outcome the ordered replay settles), and some groups are empty."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle

pytestmark = pytest.mark.gpu

L, B = omg.LongType(), omg.BooleanType()
D128 = omg.Decimal128Type(38, 2)
SUM = omg.OMNI_AGGREGATION_TYPE_SUM
M64 = (1 << 64) - 1
BIG = 4 * 10**37


def _to128(vals):
    out = np.zeros((len(vals), 2), dtype=np.uint64)
    for i, v in enumerate(vals):
        out[i, 0] = v & M64
        out[i, 1] = (v >> 64) & M64
    return out


def _from128(arr):
    v = (int(arr[1]) << 64) | int(arr[0])
    return v - (1 << 128) if v >> 127 else v


def _raw_data(n, groups, seed):
    rng = np.random.default_rng(seed)
    key = rng.integers(0, groups, n).astype(np.int64)
    vals = [int(x) for x in rng.integers(-10**12, 10**12, n)]
    for i in range(n):
        g = int(key[i])
        if g % 11 == 0:    # large values: overflow in a partial, or only on a prefix of the merge
            vals[i] = BIG if (i + g) % 3 else -BIG
        elif g % 13 == 0:  # balanced large values: exact total in range, the running sum may leave it
            vals[i] = BIG if i % 2 else -BIG
    nulls = rng.random(n) < 0.05
    nulls[key % 7 == 0] = True  # groups without values
    return key, vals, nulls


def _partial_expected(key, vals, nulls):
    """(sum or None, isEmpty) per group of one partial operator's rows, from the single-stage oracle."""
    keys, _, ovals, onulls = oracle.hashagg(
        [key], [oracle.T_LONG], [None],
        [dict(func=oracle.F_SUM, col=_to128(vals), in_type=oracle.T_DEC128, out_type=oracle.T_DEC128, nulls=nulls),
         dict(func=oracle.F_COUNT_COL, col=_to128(vals), in_type=oracle.T_DEC128, out_type=oracle.T_LONG,
              nulls=nulls)], overflow_as_null=True)
    out = {}
    for i in range(len(keys[0])):
        k = int(keys[0][i])
        if int(ovals[1][i]) == 0:
            out[k] = (0, True)
        elif onulls[0][i]:
            out[k] = (None, False)
        else:
            out[k] = (_from128(ovals[0][i]), False)
    return out


def _rows(cols, nkeys=1):
    """{key: (sum or None, isEmpty or None)} of (key, sum[, isEmpty]) output columns."""
    out = {}
    for i in range(len(cols[0][0])):
        k = int(cols[0][0][i])
        s = None if cols[1][1][i] else _from128(cols[1][0][i])
        e = bool(cols[2][0][i]) if len(cols) > 2 else None
        out[k] = (s, e)
    return out


def _drain_columns(op):
    parts = [omg.batch_to_numpy(b) for b in op.drain()]
    return None if not parts else [(np.concatenate([p[c][0] for p in parts]), np.concatenate([p[c][1] for p in parts]))
                                   for c in range(len(parts[0]))]


def _partials(key, vals, nulls, splits, strategy=None):
    """Run one partial operator per row range; returns [(partial batch handles, their columns)]."""
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[D128]], [[D128, B]], [SUM],
                                             output_partials=[True])
    out = []
    try:
        for s, e in splits:
            op = fac.create_operator()
            if strategy is not None:
                op.set_agg_strategy(strategy, 0)
            for b0 in range(s, e, 4096):
                b1 = min(e, b0 + 4096)
                op.add_input(omg.make_batch([L, D128], [key[b0:b1], _to128(vals[b0:b1])], [None, nulls[b0:b1]]))
            batches = op.drain()
            op.delete()
            out.append(batches)
    finally:
        fac.close()
    return out


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL])
def test_partial_then_final_decimal_sum(gpu, strategy):
    n, groups = 30_000, 500
    key, vals, nulls = _raw_data(n, groups, 1)
    splits = [(0, 9000), (9000, 21000), (21000, n)]
    parts = _partials(key, vals, nulls, splits, strategy)
    # Every partial operator's (sum, isEmpty) against the oracle.
    fed = []  # partial rows in the order the final operator receives them
    for (s, e), batches in zip(splits, parts):
        got = {}
        for b in batches:
            c = omg.batch_to_numpy(b)
            got.update(_rows(c))
            for i in range(len(c[0][0])):
                fed.append((int(c[0][0][i]), 0 if c[1][1][i] else _from128(c[1][0][i]), bool(c[1][1][i]),
                            bool(c[2][0][i])))
        assert got == _partial_expected(key[s:e], vals[s:e], nulls[s:e])
    # Final stage over all partial batches, in order; overflow as NULL.
    fin = omg.HashAggregationOperatorFactory([0], [L], [[1, 2]], [[D128, B]], [[D128]], [SUM],
                                             input_raws=[False], overflow_as_null=True)
    op = fin.create_operator()
    try:
        if strategy is not None:
            op.set_agg_strategy(strategy, 0)
        for batches in parts:
            for b in batches:
                op.add_input(b)
        cols = _drain_columns(op)
    finally:
        op.delete()
        fin.close()
    want = oracle.decimal_sum_merge(*zip(*fed))
    got = _rows(cols)
    assert set(got) == set(want)
    kinds = {"overflow": 0, "empty": 0, None: 0}
    for k, (v, flag) in want.items():
        kinds[flag] += 1
        assert got[k][0] == v, (k, got[k], want[k])
    assert kinds["overflow"] > 0 and kinds["empty"] > 0 and kinds[None] > 0


def test_intermediate_stage_keeps_the_pair(gpu):
    n = 20_000
    key, vals, nulls = _raw_data(n, 300, 2)
    splits = [(0, 5000), (5000, 12000), (12000, n)]
    parts = _partials(key, vals, nulls, splits)
    fed = []
    for batches in parts:
        for b in batches:
            c = omg.batch_to_numpy(b)
            for i in range(len(c[0][0])):
                fed.append((int(c[0][0][i]), 0 if c[1][1][i] else _from128(c[1][0][i]), bool(c[1][1][i]),
                            bool(c[2][0][i])))
    mid = omg.HashAggregationOperatorFactory([0], [L], [[1, 2]], [[D128, B]], [[D128, B]], [SUM],
                                             input_raws=[False], output_partials=[True])
    op = mid.create_operator()
    try:
        for batches in parts:
            for b in batches:
                op.add_input(b)
        cols = _drain_columns(op)
    finally:
        op.delete()
        mid.close()
    assert _rows(cols) == oracle.decimal_sum_merge(*zip(*fed), partial=True)


def test_final_overflow_raises_unless_overflow_as_null(gpu):
    key = np.zeros(4, dtype=np.int64)
    sums = _to128([BIG, BIG, BIG, 0])  # 1.2e38 > 10^38 - 1 on the third row
    empty = np.array([0, 0, 0, 1], dtype=np.int8)
    fin = omg.HashAggregationOperatorFactory([0], [L], [[1, 2]], [[D128, B]], [[D128]], [SUM], input_raws=[False])
    op = fin.create_operator()
    try:
        op.add_input(omg.make_batch([L, D128, B], [key, sums, empty]))
        with pytest.raises(omg.OmgError):
            op.drain()
    finally:
        op.delete()
        fin.close()
