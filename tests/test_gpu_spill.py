"""Aggregation spill on the GPU: with a device-memory budget smaller than the group table, the
operator hash-partitions its rows into pinned host memory and aggregates one partition at a time
(the role of the reference's spill path, group_aggregation.cpp:1034-1475).  Partitions hold
disjoint groups, so results must equal the oracle's exactly (doubles within 1e-12 * max(|exact|,
sum|x|) of the correctly rounded sum) and equal the unspilled run's."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, split

pytestmark = pytest.mark.gpu

L, D, I = omg.LongType(), omg.DoubleType(), omg.IntType()
SUM, CNT, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                           omg.OMNI_AGGREGATION_TYPE_AVG, omg.OMNI_AGGREGATION_TYPE_MAX,
                           omg.OMNI_AGGREGATION_TYPE_MIN)


def _run(fac_args, columns, types, nulls, budget, batch=8192, device_input=False, strategy=None):
    fac = omg.HashAggregationOperatorFactory(*fac_args[:6], **fac_args[6] if len(fac_args) > 6 else {})
    op = fac.create_operator()
    try:
        if budget:
            op.set_spill(True, budget)
        if strategy is not None:
            op.set_agg_strategy(strategy, 0)
        for s, e in split(len(columns[0]), [batch, 3001]):
            b = omg.make_batch(types, [c[s:e] for c in columns], [None if m is None else m[s:e] for m in nulls])
            if device_input:
                d = omg.batch_to_device(b)
                omg.free_batch(b)
                b = d
            op.add_input(b)
        outs = op.drain()
        assert op.get_status() == omg.OMNI_STATUS_FINISHED
        spilled = op.spilled_bytes()
        keys = op.get_hashmap_unique_keys()
    finally:
        op.delete()
        fac.close()
    cols = None
    for b in outs:
        c = omg.batch_to_numpy(b)
        omg.free_batch(b)
        cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                       for a, x in zip(cols, c)]
    return cols, spilled, keys


def _cfg_like(n, groups, seed):
    rng = np.random.default_rng(seed)
    uniq = rng.integers(-2**62, 2**62, groups, dtype=np.int64)
    key = uniq[rng.integers(0, groups, n)]
    km = rng.random(n) < 0.01
    v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    m1 = rng.random(n) < 0.02
    v2 = rng.random(n)
    m2 = rng.random(n) < 0.02
    return key, km, v1, m1, v2, m2


FAC = ([0], [L], [[1], [1], [1], [1], [2], [2]], [[L], [L], [L], [L], [D], [D]], [[L], [L], [L], [L], [D], [D]],
       [SUM, CNT, MIN, MAX, SUM, AVG])


def _oracle_check(cols, key, km, v1, m1, v2, m2):
    ora = oracle.hashagg(
        [key], [oracle.T_LONG], [km],
        [dict(func=f, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1)
         for f in (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_MIN, oracle.F_MAX)] +
        [dict(func=f, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2)
         for f in (oracle.F_SUM, oracle.F_AVG)])
    ex_s = exact_by_key([key], [km], v2, ~m2)
    ex_a = exact_by_key([key], [km], v2, ~m2, divide_by_count=True)
    assert_agg_equal(cols, ora, 1, double_aggs=(4, 5), exact={4: ex_s, 5: ex_a})


@pytest.mark.parametrize("budget_mb,device_input", [(2, False), (8, False), (2, True)])
def test_spilled_aggregation_matches_oracle(budget_mb, device_input):
    key, km, v1, m1, v2, m2 = _cfg_like(1 << 20, 150_000, budget_mb + device_input)
    cols, spilled, keys = _run(FAC, [key, v1, v2], [L, L, D], [km, m1, m2], budget_mb << 20,
                               device_input=device_input)
    assert spilled > 0
    assert keys == len(cols[0][0])
    _oracle_check(cols, key, km, v1, m1, v2, m2)


def test_budget_above_the_table_does_not_spill_and_results_agree():
    key, km, v1, m1, v2, m2 = _cfg_like(300_000, 20_000, 7)
    big, spilled_big, _ = _run(FAC, [key, v1, v2], [L, L, D], [km, m1, m2], 1 << 34)
    small, spilled_small, _ = _run(FAC, [key, v1, v2], [L, L, D], [km, m1, m2], 1 << 18)
    assert spilled_big == 0 and spilled_small > 0
    _oracle_check(big, key, km, v1, m1, v2, m2)
    _oracle_check(small, key, km, v1, m1, v2, m2)


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_GLOBAL, omg.AGG_STRATEGY_PARTITIONED])
def test_spilled_two_column_keys(strategy):
    rng = np.random.default_rng(5 + strategy)
    n = 400_000
    k1 = rng.integers(0, 300, n).astype(np.int32)
    k2 = rng.integers(0, 400, n).astype(np.int64)
    m = [rng.random(n) < 0.02 for _ in range(3)]
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    fac = ([0, 1], [I, L], [[2], [2], [2]], [[L]] * 3, [[L]] * 3, [SUM, MIN, MAX])
    cols, spilled, _ = _run(fac, [k1, k2, v], [I, L, L], m, 1 << 20, strategy=strategy)
    assert spilled > 0
    ora = oracle.hashagg([k1, k2], [oracle.T_INT, oracle.T_LONG], [m[0], m[1]],
                         [dict(func=f, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m[2])
                          for f in (oracle.F_SUM, oracle.F_MIN, oracle.F_MAX)])
    assert_agg_equal(cols, ora, 2)


def test_spilled_partial_stage_feeds_a_final_stage():
    """A spilled partial aggregation's output batches, merged by an unspilled final stage, equal
    the single-stage result."""
    key, km, v1, m1, _, _ = _cfg_like(500_000, 60_000, 11)
    partial = ([0], [L], [[1], [1]], [[L], [L]], [[L], [L]], [SUM, CNT], dict(output_partials=[True, True]))
    pcols, spilled, _ = _run(partial, [key, v1], [L, L], [km, m1], 1 << 20)
    assert spilled > 0
    final = ([0], [L], [[1], [2]], [[L], [L]], [[L], [L]], [SUM, CNT], dict(input_raws=[False, False]))
    fcols, _, _ = _run(final, [pcols[0][0], pcols[1][0], pcols[2][0]], [L, L, L],
                       [pcols[0][1], pcols[1][1], pcols[2][1]], 0)
    ora = oracle.hashagg([key], [oracle.T_LONG], [km],
                         [dict(func=f, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1)
                          for f in (oracle.F_SUM, oracle.F_COUNT_COL)])
    assert_agg_equal(fcols, ora, 1)


@pytest.mark.parametrize("device_input", [False, True])
def test_spilled_order_dependent_sums_keep_row_order(device_input):
    """Generic policy int64 SUM with sticky overflow (overflow -> NULL): whether a group overflows
    depends on the order of its rows, so the spill partitions keep each group's rows in input
    order; against the oracle folding the rows in order, and the unspilled run."""
    rng = np.random.default_rng(71)
    n, groups = 200_000, 3000
    big = 2**62
    key = rng.integers(0, groups, n).astype(np.int64) * 7919
    val = np.where(rng.random(n) < 0.5, rng.choice(np.array([big, -big], dtype=np.int64), n),
                   rng.integers(-10**6, 10**6, n, dtype=np.int64))
    args = ([0], [L], [[1]], [[L]], [[L]], [SUM], {"overflow_as_null": True})
    omg.set_policy(omg.POLICY_GENERIC)
    try:
        got, spilled, _ = _run(args, [key, val], [L, L], [None, None], 64 << 10, device_input=device_input)
        plain, spilled0, _ = _run(args, [key, val], [L, L], [None, None], 0)
        ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                             [dict(func=oracle.F_SUM, col=val, in_type=oracle.T_LONG, out_type=oracle.T_LONG)],
                             policy=1, overflow_as_null=True)
    finally:
        omg.set_policy(omg.POLICY_SPARK)
    assert spilled > 0 and spilled0 == 0
    assert_agg_equal(got, ora, 1)
    assert_agg_equal(plain, ora, 1)
    nulls = int(got[1][1].sum())
    assert 0 < nulls < groups  # both outcomes occur


@pytest.mark.parametrize("device_input", [False, True])
def test_spilled_varchar_keys_equal_the_unspilled_run(device_input):
    """VARCHAR group-by keys spill as their dictionary ids (the operator's string dictionary takes
    every pending row first); the partitions aggregate the ids and their key columns come back as
    strings.  Equal, row for row, to the unspilled run (itself checked against the oracle by the
    VARCHAR aggregation tests), NULL keys and empty strings included."""
    rng = np.random.default_rng(72)
    n = 120_000
    pool = [b""] + [bytes(rng.integers(97, 123, int(rng.integers(1, 20)), dtype=np.uint8)) for _ in range(6000)]
    keys = np.array([pool[i] for i in rng.integers(0, len(pool), n)], dtype=object)
    km = rng.random(n) < 0.01
    v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    m1 = rng.random(n) < 0.05
    v2 = rng.random(n)
    V = omg.VarcharType(24)
    args = ([0], [V], [[1], [1], [1], [1], [2]], [[L], [L], [L], [L], [D]], [[L], [L], [L], [L], [D]],
            [SUM, CNT, MIN, MAX, AVG])
    got, spilled, _ = _run(args, [keys, v1, v2], [V, L, D], [km, m1, None], 32 << 10, device_input=device_input)
    plain, spilled0, _ = _run(args, [keys, v1, v2], [V, L, D], [km, m1, None], 0)
    assert spilled > 0 and spilled0 == 0

    def rows(cols):
        out = {}
        for i in range(len(cols[0][0])):
            k = None if cols[0][1][i] else bytes(cols[0][0][i])
            out[k] = tuple(None if c[1][i] else (float(c[0][i]) if c[0].dtype.kind == "f" else int(c[0][i]))
                           for c in cols[1:])
        return out

    a, b = rows(got), rows(plain)
    assert set(a) == set(b) and len(a) > 5000
    for k in a:
        assert a[k][:4] == b[k][:4]
        assert (a[k][4] is None) == (b[k][4] is None)
        if a[k][4] is not None:
            assert abs(a[k][4] - b[k][4]) <= 1e-12 * max(1.0, abs(b[k][4]))
