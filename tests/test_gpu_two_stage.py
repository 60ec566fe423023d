"""Two-stage (partial -> final) HashAggregation on the GPU.

A partial stage (outputPartial) emits per-group intermediate columns; a final stage (inputRaw =
false) merges them (group_aggregation.cpp:1182-1218).  SUM/MIN/MAX partials are plain results,
COUNT partials are summed, and an AVG partial is the pair (double sum, long count) that the
final stage divides.  The reference passes the AVG pair as one container column; the flat form
here passes it as two adjacent columns, the final AVG reading both."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, split

pytestmark = pytest.mark.gpu

SUM, CNT, CNT_ALL, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                                    omg.OMNI_AGGREGATION_TYPE_COUNT_ALL, omg.OMNI_AGGREGATION_TYPE_AVG,
                                    omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_MIN)
L, D = omg.LongType(), omg.DoubleType()


def _batches(types, cols, nulls, sizes):
    n = len(cols[0])
    return [omg.make_batch(types, [c[s:e] for c in cols],
                           None if nulls is None else [None if m is None else m[s:e] for m in nulls])
            for s, e in split(n, sizes)]


def _run(fac, batches, strategy=None):
    """Feed batches (ownership passes) and return the output batches."""
    op = fac.create_operator()
    try:
        if strategy is not None:
            op.set_agg_strategy(strategy, 0)
        for b in batches:
            op.add_input(b)
        outs = op.drain()
        assert op.get_status() == omg.OMNI_STATUS_FINISHED
    finally:
        op.delete()
    return outs


def _columns(batches):
    cols = None
    for b in batches:
        c = omg.batch_to_numpy(b)
        omg.free_batch(b)
        cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                       for a, x in zip(cols, c)]
    return cols


def test_verify_correctness_two_stage_kat():
    """Flat form of aggregation_test.cpp:544-631: keys (j % 10, j % 10), all values 1, two partial
    operators over 10 batches x 2000 rows each, one final operator; every group has SUM 4000,
    AVG 1.0, COUNT 4000, MIN 1, MAX 1."""
    funcs = [SUM, AVG, CNT, MIN, MAX]
    keys = np.arange(2000, dtype=np.int64) % 10
    ones = np.ones(2000, dtype=np.int64)
    part = omg.HashAggregationOperatorFactory([0, 1], [L, L], [[2], [3], [4], [5], [6]], [[L]] * 5,
                                              [[L], [D, L], [L], [L], [L]], funcs, output_partials=[True] * 5)
    partials = []
    for _ in range(2):
        batches = [omg.make_batch([L] * 7, [keys, keys, ones, ones, ones, ones, ones]) for _ in range(10)]
        outs = _run(part, batches)
        assert len(outs) == 1  # one output batch per partial operator, as the reference expects
        partials += outs
    part.close()
    # partial columns: k0 k1 | sum | avg sum, avg count | count | min | max
    fin = omg.HashAggregationOperatorFactory([0, 1], [L, L], [[2], [3, 4], [5], [6], [7]],
                                             [[L], [D, L], [L], [L], [L]], [[L], [D], [L], [L], [L]], funcs,
                                             input_raws=[False] * 5)
    cols = _columns(_run(fin, partials))
    fin.close()
    assert len(cols) == 7
    order = np.argsort(cols[0][0])
    assert np.array_equal(cols[0][0][order], np.arange(10)) and np.array_equal(cols[1][0][order], np.arange(10))
    assert np.all(cols[2][0] == 4000) and np.all(cols[3][0] == 1.0) and np.all(cols[4][0] == 4000)
    assert np.all(cols[5][0] == 1) and np.all(cols[6][0] == 1)
    assert not any(c[1].any() for c in cols)


def test_verify_distinct_correctness_two_stage_kat():
    """aggregation_test.cpp:1381-1460 with its aggregation masks restated as NULL values (a row
    whose mask is false does not reach that aggregator, exactly like a NULL value): one group,
    COUNT 3, SUM 6, AVG 5.0, MAX 4, MIN 1 after partial -> final."""
    key = np.ones(4, dtype=np.int64)
    data = [np.array(v, dtype=np.int64) for v in ([10, 20, 10, 30], [1, 1, 2, 3], [3, 5, 5, 7], [4, 2, 1, 2],
                                                   [4, 2, 1, 2])]
    masks = [np.array(m) for m in ([1, 1, 0, 1], [1, 0, 1, 1], [1, 1, 0, 1], [1, 1, 1, 0], [1, 1, 1, 0])]
    nulls = [None] + [m == 0 for m in masks]
    funcs = [CNT, SUM, AVG, MAX, MIN]
    part = omg.HashAggregationOperatorFactory([0], [L], [[1], [2], [3], [4], [5]], [[L]] * 5,
                                              [[L], [L], [D, L], [L], [L]], funcs, output_partials=[True] * 5)
    outs = _run(part, [omg.make_batch([L] * 6, [key] + data, nulls)])
    part.close()
    fin = omg.HashAggregationOperatorFactory([0], [L], [[1], [2], [3, 4], [5], [6]], [[L], [L], [D, L], [L], [L]],
                                             [[L], [L], [D], [L], [L]], funcs, input_raws=[False] * 5)
    cols = _columns(_run(fin, outs))
    fin.close()
    assert [c[0].tolist() for c in cols] == [[1], [3], [6], [5.0], [4], [1]]
    assert not any(c[1].any() for c in cols)


def _random_input(n, seed):
    rng = np.random.default_rng(seed)
    pool = rng.choice(np.arange(-2**40, 2**40, 7919, dtype=np.int64), 3000, replace=False)
    key = pool[rng.integers(0, len(pool), n)]
    knull = rng.random(n) < 0.01
    key[knull] = 0
    dead = pool[:5]  # groups whose values are all NULL
    vlong = rng.integers(-2**62, 2**62, n, dtype=np.int64)  # large enough that SUM wraps (Spark policy)
    vdbl = rng.standard_normal(n) * 1e3
    vnull = (rng.random(n) < 0.1) | np.isin(key, dead)
    dnull = (rng.random(n) < 0.1) | np.isin(key, dead)
    return key, knull, vlong, vnull, vdbl, dnull, dead


@pytest.mark.parametrize("strategy", [None, omg.AGG_STRATEGY_GLOBAL, omg.AGG_STRATEGY_PARTITIONED])
def test_partial_intermediate_final_equals_single_stage(strategy):
    """Three partial operators over disjoint row ranges -> an intermediate merge (AVG stays a
    pair) -> a final operator; the result equals single-stage aggregation of all rows."""
    n = 300_000
    key, knull, vlong, vnull, vdbl, dnull, dead = _random_input(n, 11)
    types = [L, L, D]
    funcs = [SUM, CNT, CNT_ALL, MIN, MAX, AVG, AVG, SUM]
    agg_cols = [[1], [1], [], [1], [1], [2], [1], [2]]
    in_types = [[L], [L], [], [L], [L], [D], [L], [D]]
    part_out = [[L], [L], [L], [L], [L], [D, L], [D, L], [D]]
    part = omg.HashAggregationOperatorFactory([0], [L], agg_cols, in_types, part_out, funcs,
                                              output_partials=[True] * len(funcs))
    partials = []
    thirds = [(0, n // 3), (n // 3, 2 * n // 3), (2 * n // 3, n)]
    for i, (s, e) in enumerate(thirds):
        batches = _batches(types, [key[s:e], vlong[s:e], vdbl[s:e]], [knull[s:e], vnull[s:e], dnull[s:e]],
                           [4096, 1000, 3333][i:] + [4096])
        partials += _run(part, batches, strategy)
    part.close()
    # partial layout: key | sum | cnt | cnt_all | min | max | avgd sum, cnt | avgl sum, cnt | sumd
    merge_cols = [[1], [2], [3], [4], [5], [6, 7], [8, 9], [10]]
    merge_in = [[L], [L], [L], [L], [L], [D, L], [D, L], [D]]
    mid = omg.HashAggregationOperatorFactory([0], [L], merge_cols, merge_in, part_out, funcs,
                                             input_raws=[False] * len(funcs), output_partials=[True] * len(funcs))
    merged = _run(mid, partials, strategy)
    mid.close()
    fin_out = [[L], [L], [L], [L], [L], [D], [D], [D]]
    fin = omg.HashAggregationOperatorFactory([0], [L], merge_cols, merge_in, fin_out, funcs,
                                             input_raws=[False] * len(funcs))
    cols = _columns(_run(fin, merged, strategy))
    fin.close()

    T_LONG, T_DOUBLE = oracle.T_LONG, oracle.T_DOUBLE
    ora = oracle.hashagg([key], [T_LONG], [knull], [
        dict(func=SUM, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=CNT, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=CNT_ALL, col=None, out_type=T_LONG),
        dict(func=MIN, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=MAX, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=AVG, col=vdbl, in_type=T_DOUBLE, out_type=T_DOUBLE, nulls=dnull),
        dict(func=AVG, col=vlong, in_type=T_LONG, out_type=T_DOUBLE, nulls=vnull),
        dict(func=SUM, col=vdbl, in_type=T_DOUBLE, out_type=T_DOUBLE, nulls=dnull),
    ])
    exact = {5: exact_by_key([key], [knull], vdbl, ~dnull, divide_by_count=True),
             6: exact_by_key([key], [knull], vlong.astype(np.float64), ~vnull, divide_by_count=True),
             7: exact_by_key([key], [knull], vdbl, ~dnull)}
    # AVG(long) sums int64 values as doubles: each partial adds one rounding of |x| <= 2^62 per row
    # at most, covered by the Sum|x| term of the tolerance.
    assert_agg_equal(cols, ora, 1, double_aggs=(5, 6, 7), exact=exact)
    # all-NULL groups: SUM/MIN/MAX/AVG NULL, COUNT 0 after the merge (the partial AVG was (0, 0))
    rows = [i for i in range(len(cols[0][0])) if not cols[0][1][i] and cols[0][0][i] in set(dead.tolist())]
    assert len(rows) == len(dead)
    for r in rows:
        assert cols[1][1][r] and cols[4][1][r] and cols[5][1][r] and cols[6][1][r] and cols[7][1][r] and cols[8][1][r]
        assert not cols[2][1][r] and cols[2][0][r] == 0 and cols[3][0][r] > 0


def test_align_schema_restates_each_row_as_a_partial():
    """AlignSchema (group_aggregation.cpp:1182-1218 and the aggregators' ProcessAlignAggSchema):
    keys copied, SUM/MIN/MAX partials are the value (NULL kept, int widened to the output type),
    COUNT(col) 1 or 0, COUNT(*) 1, AVG (double(value) or 0, 1 or 0)."""
    rng = np.random.default_rng(4)
    n = 10_000
    key = rng.integers(-5, 5, n).astype(np.int64)
    knull = rng.random(n) < 0.05
    vint = rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
    inull = rng.random(n) < 0.2
    vdbl = rng.standard_normal(n)
    dnull = rng.random(n) < 0.2
    I = omg.IntType()
    funcs = [SUM, CNT, CNT_ALL, MIN, MAX, AVG, AVG, SUM]
    agg_cols = [[1], [1], [], [1], [1], [2], [1], [2]]
    in_types = [[I], [I], [], [I], [I], [D], [I], [D]]
    out_types = [[L], [L], [L], [I], [I], [D, L], [D, L], [D]]
    fac = omg.HashAggregationOperatorFactory([0], [L], agg_cols, in_types, out_types, funcs,
                                             output_partials=[True] * len(funcs))
    op = fac.create_operator()
    out = op.align_schema(omg.make_batch([L, I, D], [key, vint, vdbl], [knull, inull, dnull]))
    cols = omg.batch_to_numpy(out)
    omg.free_batch(out)
    empty = op.align_schema(omg.make_batch([L, I, D], [np.zeros(0, np.int64), np.zeros(0, np.int32),
                                                       np.zeros(0, np.float64)]))
    assert omg.batch_row_count(empty) == 0 and omg.lib().omg_batch_vector_count(empty) == 11
    omg.free_batch(empty)
    op.delete()
    fac.close()
    assert len(cols) == 11
    valid_i, valid_d = ~inull, ~dnull
    expect = [(key, knull), (vint.astype(np.int64), inull), (valid_i.astype(np.int64), None), (np.ones(n), None),
              (vint, inull), (vint, inull), (np.where(valid_d, vdbl, 0.0), None), (valid_d.astype(np.int64), None),
              (np.where(valid_i, vint.astype(np.float64), 0.0), None), (valid_i.astype(np.int64), None),
              (vdbl, dnull)]
    for j, ((gv, gm), (ev, em)) in enumerate(zip(cols, expect)):
        em = np.zeros(n, bool) if em is None else em
        assert np.array_equal(gm, em), j
        assert np.array_equal(gv[~em], np.asarray(ev)[~em]), j


@pytest.mark.parametrize("strategy", [None, omg.AGG_STRATEGY_PARTITIONED])
def test_adaptive_partial_aggregation_equals_single_stage(strategy):
    """Spark's adaptive partial aggregation: some batches are aggregated by the partial
    operator, the rest only aligned to its output schema (AlignSchema); the final stage merges
    both kinds of partial rows into the single-stage result."""
    n = 200_000
    key, knull, vlong, vnull, vdbl, dnull, dead = _random_input(n, 21)
    types = [L, L, D]
    funcs = [SUM, CNT, CNT_ALL, MIN, MAX, AVG, SUM]
    agg_cols = [[1], [1], [], [1], [1], [2], [2]]
    in_types = [[L], [L], [], [L], [L], [D], [D]]
    part_out = [[L], [L], [L], [L], [L], [D, L], [D]]
    part = omg.HashAggregationOperatorFactory([0], [L], agg_cols, in_types, part_out, funcs,
                                              output_partials=[True] * len(funcs))
    batches = _batches(types, [key, vlong, vdbl], [knull, vnull, dnull], [4096, 3000])
    aggregated = _run(part, batches[::2], strategy)
    aligner = part.create_operator()
    aligned = [aligner.align_schema(b) for b in batches[1::2]]
    aligner.delete()
    part.close()
    merge_cols = [[1], [2], [3], [4], [5], [6, 7], [8]]
    merge_in = [[L], [L], [L], [L], [L], [D, L], [D]]
    fin = omg.HashAggregationOperatorFactory([0], [L], merge_cols, merge_in, [[L], [L], [L], [L], [L], [D], [D]],
                                             funcs, input_raws=[False] * len(funcs))
    cols = _columns(_run(fin, aligned + aggregated, strategy))
    fin.close()
    T_LONG, T_DOUBLE = oracle.T_LONG, oracle.T_DOUBLE
    ora = oracle.hashagg([key], [T_LONG], [knull], [
        dict(func=SUM, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=CNT, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=CNT_ALL, col=None, out_type=T_LONG),
        dict(func=MIN, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=MAX, col=vlong, in_type=T_LONG, out_type=T_LONG, nulls=vnull),
        dict(func=AVG, col=vdbl, in_type=T_DOUBLE, out_type=T_DOUBLE, nulls=dnull),
        dict(func=SUM, col=vdbl, in_type=T_DOUBLE, out_type=T_DOUBLE, nulls=dnull),
    ])
    exact = {5: exact_by_key([key], [knull], vdbl, ~dnull, divide_by_count=True),
             6: exact_by_key([key], [knull], vdbl, ~dnull)}
    assert_agg_equal(cols, ora, 1, double_aggs=(5, 6), exact=exact)


@pytest.mark.parametrize("policy", [omg.POLICY_GENERIC, omg.POLICY_SPARK])
def test_container_avg_partial_intermediate_final(policy):
    """The reference's container-vector form of a partial AVG (average_aggregator.cpp:13-38,
    230-300): the partial emits one CONTAINER column of (double sum, long count) fields, an
    intermediate stage reads and emits containers, the final AVG reads the container; the result
    equals the flat-pair stages and single-stage AVG; AlignSchema emits the same container."""
    C_ = omg.ContainerType()
    n = 200_000
    key, knull, vlong, vnull, vdbl, dnull, dead = _random_input(n, 21)
    types = [L, L, D]
    funcs = [AVG, AVG, CNT]
    try:
        omg.set_policy(policy)
        part = omg.HashAggregationOperatorFactory([0], [L], [[2], [1], [1]], [[D], [L], [L]], [[C_], [C_], [L]], funcs,
                                                  output_partials=[True] * 3)
        partials = []
        for s, e in [(0, n // 2), (n // 2, n)]:
            batches = _batches(types, [key[s:e], vlong[s:e], vdbl[s:e]], [knull[s:e], vnull[s:e], dnull[s:e]],
                               [4096, 777])
            partials += _run(part, batches)
        # the partial output: key | container(sum, count) | container(sum, count) | count
        peek = omg.batch_to_numpy(partials[0])
        assert peek[1][0] == "container" and len(peek[1][1]) == 2 and peek[1][1][0][0].dtype == np.float64
        assert peek[1][1][1][0].dtype == np.int64 and not peek[1][1][0][1].any()
        # AlignSchema of raw rows gives the same container layout
        op = part.create_operator()
        aligned = op.align_schema(_batches(types, [key[:5000], vlong[:5000], vdbl[:5000]],
                                           [knull[:5000], vnull[:5000], dnull[:5000]], [5000])[0])
        op.delete()
        a = omg.batch_to_numpy(aligned)
        assert a[1][0] == "container" and a[2][0] == "container" and len(a) == 4
        cnt = a[1][1][1][0]
        assert set(np.unique(cnt).tolist()) <= {0, 1}
        partials.append(aligned)
        part.close()
        inter = omg.HashAggregationOperatorFactory([0], [L], [[1], [2], [3]], [[C_], [C_], [L]], [[C_], [C_], [L]],
                                                   funcs, input_raws=[False] * 3, output_partials=[True] * 3)
        mids = _run(inter, partials)
        inter.close()
        fin = omg.HashAggregationOperatorFactory([0], [L], [[1], [2], [3]], [[C_], [C_], [L]], [[D], [D], [L]],
                                                 funcs, input_raws=[False] * 3)
        cols = _columns(_run(fin, mids))
        fin.close()
    finally:
        omg.set_policy(omg.POLICY_SPARK)
    # single stage over all rows plus the AlignSchema rows counted twice
    import math
    k2 = np.concatenate([key, key[:5000]])
    kn2 = np.concatenate([knull, knull[:5000]])
    vl2, vn2 = np.concatenate([vlong, vlong[:5000]]), np.concatenate([vnull, vnull[:5000]])
    vd2, dn2 = np.concatenate([vdbl, vdbl[:5000]]), np.concatenate([dnull, dnull[:5000]])
    groups = {}
    for kk, knn, xl, xln, xd, xdn in zip(k2.tolist(), kn2.tolist(), vl2.tolist(), vn2.tolist(), vd2.tolist(),
                                         dn2.tolist()):
        g = groups.setdefault(None if knn else kk, ([], [], [0]))
        if not xdn:
            g[0].append(xd)
        if not xln:
            g[1].append(float(xl))
            g[2][0] += 1
    got = {}
    for i in range(len(cols[0][0])):
        kk = None if cols[0][1][i] else int(cols[0][0][i])
        got[kk] = (None if cols[1][1][i] else float(cols[1][0][i]), None if cols[2][1][i] else float(cols[2][0][i]),
                   int(cols[3][0][i]))
    assert set(got) == set(groups)
    for kk, (avg_d, avg_l, c) in got.items():
        ds, ls, cnt = groups[kk]
        assert c == cnt[0]
        assert (avg_d is None) == (len(ds) == 0) and (avg_l is None) == (len(ls) == 0)
        if ds:
            w = math.fsum(ds) / len(ds)
            assert abs(avg_d - w) <= 1e-12 * max(1.0, abs(w)) + 1e-12 * max(abs(x) for x in ds)
        if ls:
            w = math.fsum(ls) / len(ls)
            assert abs(avg_l - w) <= 1e-9 * max(1.0, abs(w))


def test_generic_int64_sum_partial_and_final():
    """Two-stage int64 SUM under the container-vector policy (sum_aggregator.cpp:11-57,
    :168-190): each stage is the generic sticky-overflow SUM -- a partial emits the sum, NULL for a
    group that overflowed (overflow-as-null) or had no values, and the final stage sums the partial
    sums in the order it receives them, skipping NULL rows.  Both stages equal the oracle run on
    each stage's own input; a group that overflowed in one partial drops that partial's part."""
    rng = np.random.default_rng(33)
    n = 120_000
    key = rng.integers(0, 2000, n).astype(np.int64)
    knull = rng.random(n) < 0.01
    v = rng.integers(-10**6, 10**6, n).astype(np.int64)
    big = rng.random(n) < 0.002  # a few rows near 2^62: some groups overflow, some come back
    v = np.where(big, rng.choice([2**62, -(2**62), 2**62 + 12345], n), v).astype(np.int64)
    vnull = rng.random(n) < 0.05
    aggs = lambda col, nulls: [dict(func=oracle.F_SUM, col=col, in_type=oracle.T_LONG, out_type=oracle.T_LONG,
                                    nulls=nulls)]

    def rows_of(cols):
        return {None if cols[0][1][i] else int(cols[0][0][i]): None if cols[1][1][i] else int(cols[1][0][i])
                for i in range(len(cols[0][0]))}

    def oracle_rows(k, kn, val, vn):
        keys, knulls, vals, vnulls = oracle.hashagg([k], [oracle.T_LONG], [kn], aggs(val, vn), policy=1,
                                                    overflow_as_null=True)
        return {None if knulls[0][i] else int(keys[0][i]): None if vnulls[0][i] else int(vals[0][i])
                for i in range(len(keys[0]))}

    try:
        omg.set_policy(omg.POLICY_GENERIC)
        part = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [SUM], output_partials=[True],
                                                  overflow_as_null=True)
        partials, pk, pkn, pv, pvn = [], [], [], [], []
        for s, e in [(0, n // 2), (n // 2, n)]:
            outs = _run(part, _batches([L, L], [key[s:e], v[s:e]], [knull[s:e], vnull[s:e]], [4096, 777]))
            for b in outs:
                c = omg.batch_to_numpy(b)
                pk.append(c[0][0]), pkn.append(c[0][1]), pv.append(c[1][0]), pvn.append(c[1][1])
            got = {}
            for b in outs:
                got.update(rows_of(omg.batch_to_numpy(b)))
            assert got == oracle_rows(key[s:e], knull[s:e], v[s:e], vnull[s:e])
            partials += outs
        part.close()
        fin = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [SUM], input_raws=[False],
                                                 overflow_as_null=True)
        cols = _columns(_run(fin, partials))
        fin.close()
    finally:
        omg.set_policy(omg.POLICY_SPARK)
    pk, pkn, pv, pvn = (np.concatenate(x) for x in (pk, pkn, pv, pvn))
    assert pvn.any() and not pvn.all()  # some partial sums are NULL (overflowed or empty)
    assert rows_of(cols) == oracle_rows(pk, pkn, pv, pvn)
