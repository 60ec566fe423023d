"""GPU parity of HashAggregation against the oracle (seeded inputs, sizes the oracle finishes in
seconds).  Integer, decimal, COUNT and MIN/MAX results must be bit-exact, NULLs included;
double SUM/AVG within 1e-12 * max(|exact|, sum|x|) (divided by the count for AVG) of the
correctly rounded sum."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, run_agg

pytestmark = pytest.mark.gpu

L, D, I, S = omg.LongType(), omg.DoubleType(), omg.IntType(), omg.ShortType()
SUM, CNT, CALL, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                                 omg.OMNI_AGGREGATION_TYPE_COUNT_ALL, omg.OMNI_AGGREGATION_TYPE_AVG,
                                 omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_MIN)


def _uniform_case(n, groups, seed, nulls=0.0, key_nulls=0.0):
    rng = np.random.default_rng(seed)
    uniq = rng.integers(-2**62, 2**62, groups, dtype=np.int64)
    key = uniq[rng.integers(0, groups, n)]
    v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    v2 = rng.random(n)
    m1 = rng.random(n) < nulls if nulls else None
    m2 = rng.random(n) < nulls if nulls else None
    km = rng.random(n) < key_nulls if key_nulls else None
    return key, v1, v2, km, m1, m2


def _cfg1_aggs():
    return dict(group_cols=[0], group_types=[L], aggs_cols=[[1], [1], [1], [1], [2], [2]],
                agg_in_types=[[L], [L], [L], [L], [D], [D]], agg_out_types=[[L], [L], [L], [L], [D], [D]],
                funcs=[SUM, CNT, MIN, MAX, SUM, AVG])


def _cfg1_oracle(key, km, v1, m1, v2, m2):
    return oracle.hashagg(
        [key], [oracle.T_LONG], [km],
        [dict(func=oracle.F_SUM, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_COUNT_COL, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MIN, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MAX, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_SUM, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2),
         dict(func=oracle.F_AVG, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2)])


def _check_cfg1(key, v1, v2, km, m1, m2, **kw):
    cols, ctr = run_agg(**_cfg1_aggs(), columns=[key, v1, v2], types=[L, L, D], nulls=[km, m1, m2], **kw)
    ora = _cfg1_oracle(key, km, v1, m1, v2, m2)
    valid = None if m2 is None else ~m2
    ex_sum = exact_by_key([key], [km], v2, valid)
    ex_avg = exact_by_key([key], [km], v2, valid, divide_by_count=True)
    assert_agg_equal(cols, ora, 1, double_aggs=(4, 5), exact={4: ex_sum, 5: ex_avg})
    return ctr


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL])
def test_uniform_keys_config1_shape(gpu, strategy):
    key, v1, v2, km, m1, m2 = _uniform_case(300_000, 10_000, 1)
    _check_cfg1(key, v1, v2, km, m1, m2, strategy=strategy)


def test_uniform_keys_device_resident_input(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(200_000, 3_000, 2)
    _check_cfg1(key, v1, v2, km, m1, m2, device_input=True, batch_sizes=(200_000,))


def test_nulls_in_keys_and_values(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(150_000, 500, 3, nulls=0.02, key_nulls=0.01)
    _check_cfg1(key, v1, v2, km, m1, m2, batch_sizes=(4096, 1000, 777))


def test_all_null_values_give_null_aggregates(gpu):
    n = 5000
    key = np.arange(n, dtype=np.int64) % 7
    v1 = np.arange(n, dtype=np.int64)
    v2 = np.ones(n)
    m1 = np.ones(n, bool)
    m2 = np.where(key == 3, True, False)
    _check_cfg1(key, v1, v2, None, m1, m2)


def test_high_cardinality_forces_exact_resize(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(400_000, 250_000, 4)
    ctr = _check_cfg1(key, v1, v2, km, m1, m2, strategy=omg.AGG_STRATEGY_GLOBAL)
    assert ctr["resizes"] >= 1
    assert ctr["groups"] > 150_000


def test_high_cardinality_with_capacity_hint_needs_no_resize(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(400_000, 250_000, 5)
    ctr = _check_cfg1(key, v1, v2, km, m1, m2, strategy=omg.AGG_STRATEGY_GLOBAL, capacity_hint=300_000)
    assert ctr["resizes"] == 0


def test_smem_path_high_cardinality_spills(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(500_000, 300_000, 6)
    _check_cfg1(key, v1, v2, km, m1, m2, strategy=omg.AGG_STRATEGY_SMEM)


def test_skewed_keys(gpu):
    rng = np.random.default_rng(7)
    n = 300_000
    key = (rng.zipf(1.3, n) % 50_000).astype(np.int64)
    v1 = rng.integers(-10**9, 10**9, n, dtype=np.int64)
    v2 = rng.standard_normal(n)
    _check_cfg1(key, v1, v2, None, None, None)


def test_sentinel_and_extreme_keys(gpu):
    key = np.array([np.iinfo(np.int64).min, np.iinfo(np.int64).max, 0, -1, np.iinfo(np.int64).min, 0] * 100,
                   dtype=np.int64)
    v1 = np.arange(len(key), dtype=np.int64)
    v2 = np.linspace(-1, 1, len(key))
    _check_cfg1(key, v1, v2, None, None, None)


def test_spark_long_sum_wraps(gpu):
    n = 3000
    key = np.arange(n, dtype=np.int64) % 3
    v = np.full(n, 9223372036854774807, dtype=np.int64)
    cols, _ = run_agg([0], [L], [[1]], [[L]], [[L]], [SUM], [key, v], [L, L])
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_SUM, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)])
    assert_agg_equal(cols, ora, 1)


@pytest.mark.parametrize("as_null", [True, False])
def test_generic_policy_sticky_overflow_order_dependent(gpu, as_null):
    """Generic policy: int64 SUM overflow is checked on every row-ordered prefix and sticky.
    Group 0 overflows on a prefix and comes back into range (-> overflow); group 1 has the same
    values in an order whose prefixes stay in range (-> exact sum)."""
    big = 2**62
    k = [0, 0, 0, 0, 1, 1, 1, 1, 2, 2]
    v = [big, big, -big, -big, big, -big, big, -big, 5, 7]
    key = np.array(k * 50, dtype=np.int64)
    val = np.array(v * 50, dtype=np.int64)
    # Keep group 1 in range by interleaving; group 0 overflows already at its second row.
    omg.set_policy(omg.POLICY_GENERIC)
    try:
        ora_kw = dict(policy=1, overflow_as_null=as_null)
        aggs = [dict(func=oracle.F_SUM, col=val, in_type=oracle.T_LONG, out_type=oracle.T_LONG)]
        if as_null:
            cols, ctr = run_agg([0], [L], [[1]], [[L]], [[L]], [SUM], [key, val], [L, L], batch_sizes=(7, 13),
                                overflow_as_null=True)
            ora = oracle.hashagg([key], [oracle.T_LONG], [None], aggs, **ora_kw)
            assert_agg_equal(cols, ora, 1)
            assert ctr["ordered_groups"] >= 1
        else:
            with pytest.raises(OverflowError):
                oracle.hashagg([key], [oracle.T_LONG], [None], aggs, **ora_kw)
            with pytest.raises(omg.OmgError) as ei:
                run_agg([0], [L], [[1]], [[L]], [[L]], [SUM], [key, val], [L, L], overflow_as_null=False)
            assert ei.value.status == -5
    finally:
        omg.set_policy(omg.POLICY_SPARK)


def test_generic_policy_in_range_sums(gpu):
    rng = np.random.default_rng(9)
    n = 100_000
    key = rng.integers(0, 1000, n).astype(np.int64)
    val = rng.integers(-2**40, 2**40, n, dtype=np.int64)
    omg.set_policy(omg.POLICY_GENERIC)
    try:
        cols, _ = run_agg([0], [L], [[1], [1]], [[L], [L]], [[L], [D]], [SUM, AVG], [key, val], [L, L])
        ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                             [dict(func=oracle.F_SUM, col=val, in_type=oracle.T_LONG, out_type=oracle.T_LONG),
                              dict(func=oracle.F_AVG, col=val, in_type=oracle.T_LONG, out_type=oracle.T_DOUBLE)],
                             policy=1)
        ex = exact_by_key([key], [None], val.astype(np.float64), None, divide_by_count=True)
        assert_agg_equal(cols, ora, 1, double_aggs=(1,), exact={1: ex})
    finally:
        omg.set_policy(omg.POLICY_SPARK)


def test_decimal64_sum_to_decimal128_with_rescale_and_nulls(gpu):
    rng = np.random.default_rng(10)
    n = 200_000
    key = rng.integers(0, 2000, n).astype(np.int64)
    dec = rng.integers(-10**9, 10**9, n, dtype=np.int64)
    m = rng.random(n) < 0.02
    d64 = omg.Decimal64Type(18, 2)
    d128 = omg.Decimal128Type(38, 4)
    cols, _ = run_agg([0], [L], [[1], [1]], [[d64], [d64]], [[d128], [L]], [SUM, CNT], [key, dec], [L, d64],
                      nulls=[None, m])
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_SUM, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_DEC128, nulls=m,
                               rescale=2),
                          dict(func=oracle.F_COUNT_COL, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_LONG,
                               nulls=m)])
    assert_agg_equal(cols, ora, 1)


@pytest.mark.parametrize("as_null", [True, False])
def test_decimal128_sum_overflow(gpu, as_null):
    big = 10**38 - 1
    vals = np.array([[big & (2**64 - 1), big >> 64]] * 3 + [[5, 0]] * 3, dtype=np.uint64)
    key = np.array([0, 0, 0, 1, 1, 1], dtype=np.int64)
    d = omg.Decimal128Type(38, 0)
    aggs = [dict(func=oracle.F_SUM, col=vals, in_type=oracle.T_DEC128, out_type=oracle.T_DEC128)]
    if as_null:
        cols, _ = run_agg([0], [L], [[1]], [[d]], [[d]], [SUM], [key, vals], [L, d], overflow_as_null=True)
        ora = oracle.hashagg([key], [oracle.T_LONG], [None], aggs, overflow_as_null=True)
        assert_agg_equal(cols, ora, 1)
        gi = {int(k): i for i, k in enumerate(cols[0][0])}
        assert cols[1][1][gi[0]] and not cols[1][1][gi[1]]
    else:
        with pytest.raises(omg.OmgError) as ei:
            run_agg([0], [L], [[1]], [[d]], [[d]], [SUM], [key, vals], [L, d], overflow_as_null=False)
        assert ei.value.status == -5


def test_composite_int32_int64_key_with_nulls(gpu):
    rng = np.random.default_rng(11)
    n = 200_000
    pairs = rng.integers(0, 5000, n)
    k1 = (pairs % 71).astype(np.int32)
    k2 = (pairs * 2654435761 % 1000003).astype(np.int64)
    km1 = rng.random(n) < 0.01
    km2 = rng.random(n) < 0.01
    v = rng.standard_normal(n)
    vm = rng.random(n) < 0.02
    cols, _ = run_agg([0, 1], [I, L], [[2], [], [2]], [[D], [], [D]], [[D], [L], [D]], [SUM, CALL, AVG],
                      [k1, k2, v], [I, L, D], nulls=[km1, km2, vm])
    ora = oracle.hashagg([k1, k2], [oracle.T_INT, oracle.T_LONG], [km1, km2],
                         [dict(func=oracle.F_SUM, col=v, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=vm),
                          dict(func=oracle.F_COUNT_ALL, col=None, out_type=oracle.T_LONG),
                          dict(func=oracle.F_AVG, col=v, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=vm)])
    ex_s = exact_by_key([k1, k2], [km1, km2], v, ~vm)
    ex_a = exact_by_key([k1, k2], [km1, km2], v, ~vm, divide_by_count=True)
    assert_agg_equal(cols, ora, 2, double_aggs=(0, 2), exact={0: ex_s, 2: ex_a})


def test_two_long_keys_verify_correctness_shape(gpu):
    """Single-stage form of the reference's verify_correctness (aggregation_test.cpp:544-730):
    keys (j%10, j%10), SUM/AVG/COUNT/MIN/MAX of ones over 20 batches of 2000 rows."""
    rows = 2000
    j = np.tile(np.arange(rows) % 10, 20).astype(np.int64)
    ones = np.ones(len(j), dtype=np.int64)
    cols, _ = run_agg([0, 1], [L, L], [[2], [3], [4], [5], [6]], [[L]] * 5, [[L], [D], [L], [L], [L]],
                      [SUM, AVG, CNT, MIN, MAX], [j, j, ones, ones, ones, ones, ones], [L] * 7, batch_sizes=(rows,))
    assert len(cols[0][0]) == 10
    for i in range(10):
        assert cols[0][0][i] == cols[1][0][i]
        assert cols[2][0][i] == 4000 and cols[3][0][i] == 1.0 and cols[4][0][i] == 4000
        assert cols[5][0][i] == 1 and cols[6][0][i] == 1


def test_double_min_max_special_values(gpu):
    vals = np.array([np.nan, 1.5, -np.inf, np.inf, -0.0, 2.0, np.nan, 7.0, np.inf, -3.0], dtype=np.float64)
    key = np.array([0, 0, 0, 1, 1, 1, 2, 2, 3, 3], dtype=np.int64)
    cols, _ = run_agg([0], [L], [[1], [1]], [[D], [D]], [[D], [D]], [MIN, MAX], [key, vals], [L, D])
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_MIN, col=vals, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE),
                          dict(func=oracle.F_MAX, col=vals, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE)])
    assert_agg_equal(cols, ora, 1)


@pytest.mark.parametrize("ktype", ["int", "short"])
def test_narrow_key_types(gpu, ktype):
    rng = np.random.default_rng(12)
    n = 50_000
    t, dt = (I, np.int32) if ktype == "int" else (S, np.int16)
    key = rng.integers(-300, 300, n).astype(dt)
    v = rng.integers(-100, 100, n).astype(np.int32)
    cols, _ = run_agg([0], [t], [[1], [1], [1]], [[I], [I], [I]], [[L], [I], [I]], [SUM, MIN, MAX], [key, v], [t, I])
    ot = oracle.T_INT if ktype == "int" else oracle.T_SHORT
    ora = oracle.hashagg([key], [ot], [None],
                         [dict(func=oracle.F_SUM, col=v, in_type=oracle.T_INT, out_type=oracle.T_LONG),
                          dict(func=oracle.F_MIN, col=v, in_type=oracle.T_INT, out_type=oracle.T_INT),
                          dict(func=oracle.F_MAX, col=v, in_type=oracle.T_INT, out_type=oracle.T_INT)])
    assert_agg_equal(cols, ora, 1)


def test_output_split_into_reference_batch_size(gpu):
    """rowsPerBatch = ceil(1 MiB / rowBytes): 56-byte rows -> at most 18725 rows per batch."""
    key, v1, v2, km, m1, m2 = _uniform_case(300_000, 60_000, 13)
    fac = omg.HashAggregationOperatorFactory(**{k: v for k, v in zip(
        ["group_by_cols", "group_input_types", "aggs_cols", "agg_input_types", "agg_output_types", "agg_func_types"],
        _cfg1_aggs().values())})
    op = fac.create_operator()
    op.add_input(omg.make_batch([L, L, D], [key, v1, v2]))
    sizes = []
    while True:
        ret, b = op.get_output()
        if not b:
            assert ret == 0
            break
        assert ret == 1
        sizes.append(omg.batch_row_count(b))
        omg.free_batch(b)
    assert op.get_status() == omg.OMNI_STATUS_FINISHED
    assert max(sizes) <= 18725 and sum(sizes) == len(np.unique(key)) and len(sizes) >= 3
    op.delete()
    fac.close()


def test_no_input_and_empty_batches(gpu):
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1]], [[L]], [[L]], [SUM])
    op = fac.create_operator()
    ret, b = op.get_output()  # no AddInput at all: returns 0, status unchanged (group_aggregation.cpp:456-458)
    assert ret == 0 and b is None and op.get_status() == omg.OMNI_STATUS_NORMAL
    op.add_input(omg.make_batch([L, L], [np.zeros(0, np.int64), np.zeros(0, np.int64)]))
    ret, b = op.get_output()
    assert ret == 0 and b is None and op.get_status() == omg.OMNI_STATUS_FINISHED
    op.delete()
    fac.close()


def test_pipeline_mode_many_small_batches(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(120_000, 2_000, 14)
    _check_cfg1(key, v1, v2, km, m1, m2, batch_sizes=(1, 17, 300, 4096), pipeline=True)


# ---- partitioned strategy: hash partitions, one shared-memory table per partition


def test_partitioned_auto_on_uniform_config1_shape(gpu):
    # AUTO sizes from the sketch (10,000 groups) and picks several partitions.
    key, v1, v2, km, m1, m2 = _uniform_case(1_000_000, 10_000, 21)
    ctr = _check_cfg1(key, v1, v2, km, m1, m2, batch_sizes=(1_000_000,))
    sz = ctr["sizing"]
    assert sz["part_bits"] >= 1, sz
    assert 8_000 <= sz["estimate"] <= 12_500, sz
    assert ctr["resizes"] == 0


def test_partitioned_forced_with_nulls_and_ragged_batches(gpu):
    key, v1, v2, km, m1, m2 = _uniform_case(400_000, 3_000, 22, nulls=0.02, key_nulls=0.01)
    ctr = _check_cfg1(key, v1, v2, km, m1, m2, strategy=omg.AGG_STRATEGY_PARTITIONED,
                      batch_sizes=(4096, 1000, 777, 65536))
    assert ctr["sizing"]["part_bits"] >= 0


@pytest.mark.parametrize("hint", [100, 20_000])
def test_partitioned_underestimate_falls_back_to_global(gpu, hint):
    # The estimate (capacity hint) is far below the real 200,000 groups: the shared tables
    # overflow into the global table, which grows; the result stays exact.
    key, v1, v2, km, m1, m2 = _uniform_case(600_000, 200_000, 23)
    ctr = _check_cfg1(key, v1, v2, km, m1, m2, strategy=omg.AGG_STRATEGY_PARTITIONED, capacity_hint=hint,
                      batch_sizes=(600_000,))
    assert ctr["resizes"] >= 1
    assert ctr["sizing"]["estimate"] == hint


def test_partitioned_composite_key_decimal_count_all_avg(gpu):
    rng = np.random.default_rng(24)
    n = 500_000
    pairs = rng.integers(0, 20_000, n)
    k1 = (pairs % 97).astype(np.int32)
    k2 = (pairs * 2654435761 % 1000003).astype(np.int64)
    km1 = rng.random(n) < 0.005
    dec = rng.integers(-10**9, 10**9, n, dtype=np.int64)
    dm = rng.random(n) < 0.02
    v = rng.standard_normal(n)
    vm = rng.random(n) < 0.02
    d64 = omg.Decimal64Type(18, 2)
    d128 = omg.Decimal128Type(38, 2)
    cols, ctr = run_agg([0, 1], [I, L], [[2], [], [3]], [[d64], [], [D]], [[d128], [L], [D]], [SUM, CALL, AVG],
                        [k1, k2, dec, v], [I, L, d64, D], nulls=[km1, None, dm, vm],
                        strategy=omg.AGG_STRATEGY_PARTITIONED, batch_sizes=(65536,))
    assert ctr["sizing"]["part_bits"] >= 1
    ora = oracle.hashagg([k1, k2], [oracle.T_INT, oracle.T_LONG], [km1, None],
                         [dict(func=oracle.F_SUM, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_DEC128, nulls=dm),
                          dict(func=oracle.F_COUNT_ALL, col=None, out_type=oracle.T_LONG),
                          dict(func=oracle.F_AVG, col=v, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=vm)])
    ex_a = exact_by_key([k1, k2], [km1, None], v, ~vm, divide_by_count=True)
    assert_agg_equal(cols, ora, 2, double_aggs=(2,), exact={2: ex_a})


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL])
def test_decimal128_sums_next_to_empty_groups(gpu, strategy):
    """Many groups whose decimal inputs are all NULL (a NULL 16-byte result written next to
    non-NULL ones, in every output position parity): each group's two result words stay its
    own.  Negative sums set the high word, positive ones leave it zero."""
    rng = np.random.default_rng(77)
    n, groups = 400_000, 150_000
    key = rng.integers(0, groups, n).astype(np.int64)
    dec = rng.integers(-10**9, 10**9, n).astype(np.int64)
    nulls = (key % 2 == 0) | (rng.random(n) < 0.02)
    D64, D128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
    cols, _ = run_agg([0], [L], [[1]], [[D64]], [[D128]], [SUM], [key, dec], [L, D64], nulls=[None, nulls],
                      strategy=strategy, batch_sizes=(65536,))
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_SUM, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_DEC128,
                               nulls=nulls)])
    assert_agg_equal(cols, ora, 1)


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_AUTO, omg.AGG_STRATEGY_SMEM, omg.AGG_STRATEGY_GLOBAL,
                                      omg.AGG_STRATEGY_PARTITIONED])
def test_decimal128_min_max(gpu, strategy):
    """MIN / MAX of decimal128 values (min_aggregator.h, MinAggregator<DECIMAL128, DECIMAL128>):
    values of both signs up to +-(10^38 - 1), equal high words with different low words, NULLs
    and all-NULL groups, bit-exact against the oracle."""
    rng = np.random.default_rng(91)
    n, groups = 200_000, 3000
    key = rng.integers(0, groups, n).astype(np.int64)
    big = 10**38 - 1
    vals = []
    for i in range(n):
        r = rng.random()
        if r < 0.3:
            v = int(rng.integers(-10**18, 10**18))
        elif r < 0.6:
            v = int(rng.integers(-2**62, 2**62)) * (1 << 64) + int(rng.integers(0, 2**63))
        else:
            v = int(rng.integers(-2**31, 2**31)) << 64 | int(rng.integers(0, 2**63)) * 2
        vals.append(max(-big, min(big, v)))
    vals[5], vals[6] = big, -big
    dec = np.array([[v & (2**64 - 1), (v >> 64) & (2**64 - 1)] for v in vals], dtype=np.uint64)
    nulls = (rng.random(n) < 0.05) | (key % 97 == 0)
    D128 = omg.Decimal128Type(38, 3)
    cols, _ = run_agg([0], [L], [[1], [1]], [[D128], [D128]], [[D128], [D128]], [MIN, MAX], [key, dec], [L, D128],
                      nulls=[None, nulls], strategy=strategy, batch_sizes=(4096, 777))
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=f, col=dec, in_type=oracle.T_DEC128, out_type=oracle.T_DEC128, nulls=nulls)
                          for f in (oracle.F_MIN, oracle.F_MAX)])
    assert_agg_equal(cols, ora, 1)
