"""Aggregation mask columns (maskColsVector) on the GPU against the oracle.

A masked aggregator sees only the rows whose BOOLEAN mask column is TRUE; a NULL mask counts as
FALSE and every row still creates its group (MaskColAggregator::ProcessGroup,
aggregator/mask_column_assistant_aggregator.h:44-53; the factory wraps an aggregator when its
mask entry is not -1, aggregation.cpp:12-18).  Checked for every aggregate kind, masked and
unmasked aggregators over the same column, groups whose rows are all masked out, all four
strategies, several batches, device input, two-stage partials and spill."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, run_agg

pytestmark = pytest.mark.gpu

L, D, B = omg.LongType(), omg.DoubleType(), omg.BooleanType()
D64, D128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
SUM, CNT, CALL, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                                 omg.OMNI_AGGREGATION_TYPE_COUNT_ALL, omg.OMNI_AGGREGATION_TYPE_AVG,
                                 omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_MIN)
NO_MASK = 0xFFFFFFFF


def _data(n, groups, seed):
    rng = np.random.default_rng(seed)
    uniq = rng.integers(-2**62, 2**62, groups, dtype=np.int64)
    gi = rng.integers(0, groups, n)
    key = uniq[gi]
    km = rng.random(n) < 0.005
    v1 = rng.integers(-10**12, 10**12, n, dtype=np.int64)
    n1 = rng.random(n) < 0.05
    v2 = rng.standard_normal(n)
    n2 = rng.random(n) < 0.05
    dec = rng.integers(-10**15, 10**15, n, dtype=np.int64)
    nd = rng.random(n) < 0.05
    m1 = (rng.random(n) < 0.6).astype(np.int8)
    m1[gi % 17 == 0] = 0  # these groups' rows never reach the m1-masked aggregators
    m1n = rng.random(n) < 0.1
    m2 = (rng.random(n) < 0.3).astype(np.int8)
    return dict(key=key, km=km, v1=v1, n1=n1, v2=v2, n2=n2, dec=dec, nd=nd, m1=m1, m1n=m1n, m2=m2)


# Columns: 0 key, 1 v1 (long), 2 v2 (double), 3 m1 (boolean, NULLs), 4 m2 (boolean), 5 dec (decimal64).
PLAN = [  # (func, input column, input type, output type, mask column or None)
    (SUM, 1, L, L, 3), (SUM, 1, L, L, None), (CNT, 1, L, L, 3), (CALL, None, None, L, 4), (CALL, None, None, L, None),
    (MIN, 1, L, L, 4), (MAX, 1, L, L, 3), (SUM, 2, D, D, 4), (AVG, 2, D, D, 3), (SUM, 5, D64, D128, 3),
    (CNT, 2, D, L, 4),
]
ORA_FUNC = {SUM: oracle.F_SUM, CNT: oracle.F_COUNT_COL, CALL: oracle.F_COUNT_ALL, AVG: oracle.F_AVG, MAX: oracle.F_MAX,
            MIN: oracle.F_MIN}
ORA_TYPE = {id(L): oracle.T_LONG, id(D): oracle.T_DOUBLE, id(D64): oracle.T_DEC64, id(D128): oracle.T_DEC128}


def _factory_args(plan):
    return dict(group_cols=[0], group_types=[L], aggs_cols=[[] if c is None else [c] for _, c, _, _, _ in plan],
                agg_in_types=[[] if t is None else [t] for _, _, t, _, _ in plan],
                agg_out_types=[[o] for _, _, _, o, _ in plan], funcs=[f for f, _, _, _, _ in plan],
                mask_cols=[NO_MASK if m is None else m for *_, m in plan])


def _oracle(d, plan):
    cols = {1: (d["v1"], d["n1"], oracle.T_LONG), 2: (d["v2"], d["n2"], oracle.T_DOUBLE),
            5: (d["dec"], d["nd"], oracle.T_DEC64)}
    masks = {3: (d["m1"].astype(bool), d["m1n"]), 4: (d["m2"].astype(bool), None)}
    aggs = []
    for f, c, _, o, m in plan:
        a = dict(func=ORA_FUNC[f], out_type=ORA_TYPE[id(o)])
        if c is not None:
            a.update(col=cols[c][0], nulls=cols[c][1], in_type=cols[c][2])
        else:
            a.update(col=None, in_type=oracle.T_LONG)
        if m is not None:
            a.update(mask=masks[m][0], mask_nulls=masks[m][1])
        aggs.append(a)
    return oracle.hashagg([d["key"]], [oracle.T_LONG], [d["km"]], aggs)


def _exact(d, plan):
    out = {}
    for j, (f, c, _, _, m) in enumerate(plan):
        if c != 2 or f not in (SUM, AVG):
            continue
        valid = ~d["n2"]
        if m == 3:
            valid &= d["m1"].astype(bool) & ~d["m1n"]
        elif m == 4:
            valid &= d["m2"].astype(bool)
        out[j] = exact_by_key([d["key"]], [d["km"]], d["v2"], valid, divide_by_count=f == AVG)
    return out


def _columns(d):
    return ([d["key"], d["v1"], d["v2"], d["m1"], d["m2"], d["dec"]], [L, L, D, B, B, D64],
            [d["km"], d["n1"], d["n2"], d["m1n"], None, d["nd"]])


def _check(d, plan=PLAN, **kw):
    columns, types, nulls = _columns(d)
    cols, _ = run_agg(**_factory_args(plan), columns=columns, types=types, nulls=nulls, **kw)
    ora = _oracle(d, plan)
    exact = _exact(d, plan)
    assert_agg_equal(cols, ora, 1, double_aggs=tuple(exact), exact=exact)
    return cols


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_AUTO, omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL,
                                      omg.AGG_STRATEGY_PARTITIONED])
def test_masked_aggregators_every_strategy(gpu, strategy):
    d = _data(60_000, 700, 1)
    cols = _check(d, strategy=strategy, batch_sizes=(4096, 1000, 7000))
    # Groups whose m1 is always FALSE exist: their masked SUM is NULL, the unmasked one is not.
    assert cols[1][1].any() and not cols[2][1][cols[1][1]].all()


def test_masked_high_cardinality_device_input(gpu):
    d = _data(200_000, 60_000, 2)
    _check(d, strategy=omg.AGG_STRATEGY_GLOBAL, device_input=True, batch_sizes=(65536,))


def test_mask_all_false_and_all_true(gpu):
    d = _data(20_000, 300, 3)
    d["m1"][:] = 0
    d["m2"][:] = 1
    d["m1n"][:] = False
    _check(d)


def test_masked_partial_stage_matches_oracle(gpu):
    """Partial (outputPartial) masked aggregators: SUM / MIN / MAX partials are the masked
    results, COUNT partials the masked counts, and AVG the masked (sum, count) pair."""
    d = _data(50_000, 900, 4)
    plan = [(SUM, 1, L, L, 3), (CNT, 1, L, L, 4), (CALL, None, None, L, 3), (MIN, 1, L, L, 3), (MAX, 1, L, L, 4)]
    columns, types, nulls = _columns(d)
    args = _factory_args(plan)
    fac = omg.HashAggregationOperatorFactory(args["group_cols"], args["group_types"], args["aggs_cols"],
                                             args["agg_in_types"], args["agg_out_types"], args["funcs"],
                                             mask_cols=args["mask_cols"], input_raws=[True] * len(plan),
                                             output_partials=[True] * len(plan))
    op = fac.create_operator()
    try:
        for s in range(0, len(d["key"]), 4096):
            op.add_input(omg.make_batch(types, [c[s:s + 4096] for c in columns],
                                        [None if m is None else m[s:s + 4096] for m in nulls]))
        cols = None
        for b in op.drain():
            c = omg.batch_to_numpy(b)
            omg.free_batch(b)
            cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                           for a, x in zip(cols, c)]
    finally:
        op.delete()
        fac.close()
    assert_agg_equal(cols, _oracle(d, plan), 1)


def test_masked_aggregation_spills(gpu):
    """The same masked plan with a tiny device budget: the partitions carry the masked inputs
    (masks already applied) and give the oracle's result."""
    d = _data(120_000, 20_000, 5)
    plan = [p for p in PLAN if p[1] != 5]  # spill refuses order-dependent (decimal) sums
    _check(d, plan=plan, spill_budget=64 * 1024)
