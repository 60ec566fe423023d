"""VARCHAR/CHAR group-by keys in HashAggregation on the GPU.

The operator aggregates a string key as the id of the string in its string dictionary and
turns ids back into strings at output time, so the group semantics must be those of the
strings themselves: equal bytes (and equal length) make one group, the empty string is a value
distinct from NULL, and the NULL key is its own group.  The oracle aggregates the same rows with
each distinct string replaced by a distinct int64 (a bijection), which gives the same groups;
GPU output keys are mapped back through the same table.  Integer results bit-exact, double
SUM/AVG within 1e-12 * max(|exact|, sum|x|) of the correctly rounded sum.

Known answers: the reference's VARCHAR and CHAR group-by tests (aggregation_test.cpp:1195-1283)
and its two-stage MIN/MAX of VARCHAR tests (:1664-1737, :1806-1890).  MIN/MAX of VARCHAR values
compare bytes as unsigned, a proper prefix first."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, exact_by_key, run_agg, split

pytestmark = pytest.mark.gpu

L, D, V = omg.LongType(), omg.DoubleType(), omg.VarcharType(64)
CHR = omg.DataType(omg.OMNI_CHAR, 0, 0, 8)
SUM, CNT, CALL, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                                 omg.OMNI_AGGREGATION_TYPE_COUNT_ALL, omg.OMNI_AGGREGATION_TYPE_AVG,
                                 omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_MIN)


def _strings(rng, n, pool, max_len=40, prefix=b""):
    lens = rng.integers(0, max_len, pool)
    words = [prefix + bytes(rng.integers(97, 123, l, dtype=np.uint8)) for l in lens]
    words[0] = b""  # the empty string is a value, distinct from NULL
    # near-duplicates: same prefix, one byte longer or different in the last byte
    for i in range(1, min(pool, 40), 2):
        words[i + 1 if i + 1 < pool else i] = words[i] + b"x"
    idx = rng.integers(0, pool, n)
    return np.array([words[i] for i in idx], dtype=object)


class Codes:
    """Bijection string -> int64 shared by the oracle input and the GPU output."""

    def __init__(self):
        self.d = {}

    def encode(self, col, mask=None):
        out = np.zeros(len(col), dtype=np.int64)
        for i, v in enumerate(col):
            if mask is not None and mask[i]:
                continue
            out[i] = self.d.setdefault(bytes(v), len(self.d) * 7919 - 10**6)
        return out

    def decode_gpu(self, values, mask):
        out = np.zeros(len(values), dtype=np.int64)
        for i, v in enumerate(values):
            if mask[i]:
                continue
            b = bytes(v)
            assert b in self.d, f"GPU produced a string never seen in the input: {b!r}"
            out[i] = self.d[b]
        return out


def _aggs(vcol):
    """SUM, COUNT, MIN, MAX of int64 column vcol; SUM, AVG of double column vcol + 1."""
    return dict(aggs_cols=[[vcol], [vcol], [vcol], [vcol], [vcol + 1], [vcol + 1]],
                agg_in_types=[[L], [L], [L], [L], [D], [D]], agg_out_types=[[L], [L], [L], [L], [D], [D]],
                funcs=[SUM, CNT, MIN, MAX, SUM, AVG])


def _oracle(keys, kmasks, v1, m1, v2, m2):
    kt = [oracle.T_LONG] * len(keys)
    return oracle.hashagg(
        keys, kt, kmasks,
        [dict(func=oracle.F_SUM, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_COUNT_COL, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MIN, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MAX, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_SUM, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2),
         dict(func=oracle.F_AVG, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=m2)])


def _check(key_cols, key_types, key_masks, v1, m1, v2, m2, **kw):
    """Aggregate (keys..., v1, v2) on the GPU and compare with the oracle over encoded keys."""
    nk = len(key_cols)
    codes = [Codes() if t.id in (omg.OMNI_VARCHAR, omg.OMNI_CHAR) else None for t in key_types]
    enc = [c.encode(k, m) if c is not None else k for c, k, m in zip(codes, key_cols, key_masks)]
    cols, ctr = run_agg(list(range(nk)), key_types, **_aggs(nk), columns=list(key_cols) + [v1, v2],
                        types=list(key_types) + [L, D], nulls=list(key_masks) + [m1, m2], **kw)
    gpu = list(cols)
    for i, c in enumerate(codes):
        if c is not None:
            gpu[i] = (c.decode_gpu(*cols[i]), cols[i][1])
    ora = _oracle(enc, list(key_masks), v1, m1, v2, m2)
    valid = None if m2 is None else ~m2
    ex_sum = exact_by_key(enc, list(key_masks), v2, valid)
    ex_avg = exact_by_key(enc, list(key_masks), v2, valid, divide_by_count=True)
    assert_agg_equal(gpu, ora, nk, double_aggs=(4, 5), exact={4: ex_sum, 5: ex_avg})
    return cols, ctr


def _values(rng, n):
    v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    v2 = rng.random(n)
    return v1, rng.random(n) < 0.02, v2, rng.random(n) < 0.02


def _count_rows(cols):
    return {(None if m else bytes(v)): int(c) for v, m, c in zip(cols[0][0], cols[0][1], cols[1][0])}


@pytest.mark.parametrize("key_type", ["varchar", "char"])
def test_reference_varchar_group_by_count(key_type):
    """aggregation_test.cpp:1195-1240 (verify_varchar_vector_correctness) and its CHAR twin:
    group by a string column, COUNT of another string column -> {"0": 3, "1": 3, "2": 2}."""
    t = V if key_type == "varchar" else CHR
    data = np.array([b"0", b"1", b"2", b"0", b"1", b"2", b"0", b"1"], dtype=object)
    cols, _ = run_agg([0], [t], [[1]], [[t]], [[L]], [CNT], [data, data.copy()], [t, t])
    assert _count_rows(cols) == {b"0": 3, b"1": 3, b"2": 2}


def _str_rows(cols, nkeys):
    """{key tuple: value tuple} with strings as bytes, NULL as None."""
    def v(col, m, i):
        return None if m[i] else (bytes(col[i]) if isinstance(col[i], (bytes, bytearray)) else int(col[i]))
    n = len(cols[0][0])
    return {tuple(v(c, m, i) for c, m in cols[:nkeys]): tuple(v(c, m, i) for c, m in cols[nkeys:])
            for i in range(n)}


def test_reference_varchar_group_by_count_min_max():
    """aggregation_test.cpp:1195-1240 in full: group by VARCHAR(1), COUNT(VARCHAR(1)),
    MIN(VARCHAR(1)), MAX(VARCHAR(4)) -> ("0", 3, "0", "6.6"), ("1", 3, "1", "5.5"), ("2", 2, "2", "4.4")."""
    d0 = np.array([b"0", b"1", b"2", b"0", b"1", b"2", b"0", b"1"], dtype=object)
    d3 = np.array([b"6.6", b"5.5", b"4.4", b"3.3", b"2.2", b"1.1", b"1.1", b"1"], dtype=object)
    V1, V4 = omg.VarcharType(1), omg.VarcharType(4)
    cols, _ = run_agg([0], [V1], [[1], [2], [3]], [[V1], [V1], [V4]], [[L], [V1], [V4]], [CNT, MIN, MAX],
                      [d0, d0.copy(), d0.copy(), d3], [V1, V1, V1, V4])
    assert _str_rows(cols, 1) == {(b"0",): (3, b"0", b"6.6"), (b"1",): (3, b"1", b"5.5"),
                                  (b"2",): (2, b"2", b"4.4")}


def _two_stage_no_group(data, masks, funcs):
    """The reference's partial -> final MIN/MAX tests without group-by columns, in flat form:
    a constant group-by column stands in for the non-grouped aggregation."""
    n = len(data[0])
    k = np.zeros(n, dtype=np.int64)
    T = omg.VarcharType(100)
    m = len(data)
    pf = omg.HashAggregationOperatorFactory([0], [L], [[i + 1] for i in range(m)], [[T]] * m, [[T]] * m, funcs,
                                            output_partials=[True] * m)
    op = pf.create_operator()
    op.add_input(omg.make_batch([L] + [T] * m, [k] + list(data), [None] + list(masks)))
    partial = op.drain()
    op.delete()
    pf.close()
    ff = omg.HashAggregationOperatorFactory([0], [L], [[i + 1] for i in range(m)], [[T]] * m, [[T]] * m, funcs,
                                            input_raws=[False] * m)
    op = ff.create_operator()
    for b in partial:
        op.add_input(b)
    outs = op.drain()
    op.delete()
    ff.close()
    assert len(outs) == 1
    cols = omg.batch_to_numpy(outs[0])
    omg.free_batch(outs[0])
    return _str_rows(cols, 1)[(0,)]


def test_reference_min_max_varchar_two_stage():
    """aggregation_test.cpp:1664-1737 (min_max_varchar): MIN over a column NULL at rows 1 and 4,
    MAX over one NULL at rows 0 and 3 -> the Aaron.Anderson and Zulma.Carter strings."""
    d0 = np.array([b"Zulma.Carter@MfvjVN43Udd95KeZ.com", b"*", b"Aaron.Anderson@0CQ4QUkBY2Q.edu",
                   b"Zulema.Ruiz@J2XvbX7.com", b"*", b"Aaron.Artis@bv.org"], dtype=object)
    d1 = np.array([b"*", b"Zulma.Carter@MfvjVN43Udd95KeZ.com", b"Aaron.Anderson@0CQ4QUkBY2Q.edu", b"*",
                   b"Zulema.Ruiz@J2XvbX7.com", b"Aaron.Artis@bv.org"], dtype=object)
    m0 = np.array([0, 1, 0, 0, 1, 0], bool)
    m1 = np.array([1, 0, 0, 1, 0, 0], bool)
    got = _two_stage_no_group([d0, d1], [m0, m1], [MIN, MAX])
    assert got == (b"Aaron.Anderson@0CQ4QUkBY2Q.edu", b"Zulma.Carter@MfvjVN43Udd95KeZ.com")


def test_reference_min_max_varchar_mix_with_nulls():
    """aggregation_test.cpp:1806-1890: MAX, MAX, MIN, MIN over columns with empty strings, the
    first two NULL at rows 4-5 and the last two at rows 0-1 -> ("", "Zulma.Carter...", "", "")."""
    e = np.array([b""] * 6, dtype=object)
    d2 = np.array([b"Zulma.Carter@MfvjVN43Udd95KeZ.com", b"*", b"", b"Zulema.Ruiz@J2XvbX7.com", b"*", b""],
                  dtype=object)
    d4 = np.array([b"*", b"", b"Aaron.Anderson@0CQ4QUkBY2Q.edu", b"", b"Zulema.R", b"Aaron.Artis@bv.org"],
                  dtype=object)
    a = np.array([0, 0, 0, 0, 1, 1], bool)
    b = np.array([1, 1, 0, 0, 0, 0], bool)
    got = _two_stage_no_group([e, d2, e.copy(), d4], [a, a, b, b], [MAX, MAX, MIN, MIN])
    assert got == (b"", b"Zulma.Carter@MfvjVN43Udd95KeZ.com", b"", b"")


def test_empty_string_null_and_prefixes_are_distinct_groups():
    keys = np.array([b"", b"a", b"ab", b"a", b"", b"ab", b"abc", b"", b"a\x00", b"a"], dtype=object)
    mask = np.zeros(len(keys), bool)
    mask[[4, 7]] = True  # two NULL keys; one empty string stays a value
    one = np.ones(len(keys), dtype=np.int64)
    cols, _ = run_agg([0], [V], [[1]], [[L]], [[L]], [SUM], [keys, one], [V, L], nulls=[mask, None])
    assert _count_rows(cols) == {b"": 1, b"a": 3, b"ab": 2, b"abc": 1, b"a\x00": 1, None: 2}


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_AUTO, omg.AGG_STRATEGY_GLOBAL, omg.AGG_STRATEGY_SMEM,
                                      omg.AGG_STRATEGY_PARTITIONED])
def test_varchar_key_matches_oracle(strategy):
    rng = np.random.default_rng(11 + strategy)
    n = 300_000
    keys = _strings(rng, n, 5000)
    km = rng.random(n) < 0.03
    _check([keys], [V], [km], *_values(rng, n), batch_sizes=(4096, 1000, 77), strategy=strategy)


@pytest.mark.parametrize("layout", ["varchar_long", "long_varchar_varchar", "char_varchar"])
def test_multi_column_keys_with_strings_match_oracle(layout):
    rng = np.random.default_rng(len(layout))
    n = 200_000
    s1 = _strings(rng, n, 300)
    s2 = _strings(rng, n, 40, max_len=8)
    num = rng.integers(-3, 3, n).astype(np.int64)
    m = [rng.random(n) < 0.02 for _ in range(3)]
    if layout == "varchar_long":
        kc, kt, km = [s1, num], [V, L], [m[0], m[1]]
    elif layout == "long_varchar_varchar":
        kc, kt, km = [num, s1, s2], [L, V, V], m
    else:
        c8 = np.array([bytes(x[:8]) for x in s2], dtype=object)
        kc, kt, km = [c8, s1], [CHR, V], [m[0], m[1]]
    _check(kc, kt, km, *_values(rng, n), batch_sizes=(4096, 333))


def test_many_batch_sets_grow_the_dictionary():
    """Small flushes: later batch sets bring new strings (dictionary grows and is rehashed) and
    repeat earlier ones (found through the stored characters)."""
    rng = np.random.default_rng(5)
    n = 120_000
    # the pool widens over the rows: strings of rows i draw from the first (i / n * 20000) words
    pool = _strings(rng, 20_000, 20_000, prefix=b"w")
    limit = np.maximum(1, (np.arange(n) * 20_000) // n)
    keys = pool[(rng.random(n) * limit).astype(np.int64)]
    km = rng.random(n) < 0.01
    omg.lib().omg_debug_set_agg_flush_rows(7000)
    try:
        _cols, ctr = _check([keys], [V], [km], *_values(rng, n), batch_sizes=(2048, 999))
    finally:
        omg.lib().omg_debug_set_agg_flush_rows(0)
    assert ctr["kernel_launches"] >= 10  # one timed aggregation launch per batch set


def test_count_of_a_varchar_value_column():
    rng = np.random.default_rng(9)
    n = 50_000
    key = rng.integers(0, 100, n).astype(np.int64)
    s = _strings(rng, n, 50)
    sm = rng.random(n) < 0.2
    cols, _ = run_agg([0], [L], [[1], [1]], [[V], [V]], [[L], [L]], [CNT, CALL], [key, s], [L, V],
                      nulls=[None, sm], batch_sizes=(4096, 1001))
    ora = oracle.hashagg([key], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_COUNT_COL, col=key, in_type=oracle.T_LONG, out_type=oracle.T_LONG,
                               nulls=sm),
                          dict(func=oracle.F_COUNT_ALL, col=key, in_type=oracle.T_LONG, out_type=oracle.T_LONG)])
    assert_agg_equal(cols, ora, 1)


def test_two_stage_with_varchar_keys_equals_single_stage():
    """Partial operators over disjoint row ranges, then a final stage over their string-keyed
    partial outputs."""
    rng = np.random.default_rng(21)
    n = 120_000
    keys = _strings(rng, n, 2000)
    km = rng.random(n) < 0.02
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    funcs = [SUM, CNT, MIN, MAX]
    partials = []
    for s, e in split(n, [40_000]):
        pf = omg.HashAggregationOperatorFactory([0], [V], [[1]] * 4, [[L]] * 4, [[L]] * 4, funcs,
                                                output_partials=[True] * 4)
        op = pf.create_operator()
        for bs, be in split(e - s, [4096]):
            op.add_input(omg.make_batch([V, L], [keys[s + bs:s + be], v[s + bs:s + be]],
                                        [km[s + bs:s + be], None]))
        partials += op.drain()
        op.delete()
        pf.close()
    ff = omg.HashAggregationOperatorFactory([0], [V], [[1], [2], [3], [4]], [[L]] * 4, [[L]] * 4, funcs,
                                            input_raws=[False] * 4)
    op = ff.create_operator()
    for b in partials:
        op.add_input(b)
    outs = op.drain()
    op.delete()
    ff.close()
    cols = None
    for b in outs:
        c = omg.batch_to_numpy(b)
        omg.free_batch(b)
        cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                       for a, x in zip(cols, c)]
    codes = Codes()
    enc = codes.encode(keys, km)
    gpu = [(codes.decode_gpu(*cols[0]), cols[0][1])] + list(cols[1:])
    ora = oracle.hashagg([enc], [oracle.T_LONG], [km],
                         [dict(func=f, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)
                          for f in (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_MIN, oracle.F_MAX)])
    assert_agg_equal(gpu, ora, 1)


def test_order_dependent_overflow_with_varchar_keys():
    """Generic policy, int64 SUM with sticky overflow: groups whose outcome depends on row order
    are replayed over the retained batches, whose keys are read through the dictionary ids of
    their own batch set."""
    big = 2**62
    k = [b"zero", b"zero", b"zero", b"zero", b"one", b"one", b"one", b"one", b"", b""]
    v = [big, big, -big, -big, big, -big, big, -big, 5, 7]
    keys = np.array(k * 50, dtype=object)
    val = np.array(v * 50, dtype=np.int64)
    omg.set_policy(omg.POLICY_GENERIC)
    omg.lib().omg_debug_set_agg_flush_rows(60)
    try:
        cols, ctr = run_agg([0], [V], [[1]], [[L]], [[L]], [SUM], [keys, val], [V, L], batch_sizes=(7, 13),
                            overflow_as_null=True)
    finally:
        omg.lib().omg_debug_set_agg_flush_rows(0)
        omg.set_policy(omg.POLICY_SPARK)
    codes = Codes()
    enc = codes.encode(keys)
    ora = oracle.hashagg([enc], [oracle.T_LONG], [None],
                         [dict(func=oracle.F_SUM, col=val, in_type=oracle.T_LONG, out_type=oracle.T_LONG)],
                         policy=1, overflow_as_null=True)
    gpu = [(codes.decode_gpu(*cols[0]), cols[0][1])] + list(cols[1:])
    assert_agg_equal(gpu, ora, 1)
    assert ctr["ordered_groups"] >= 1


def test_high_cardinality_strings():
    """2^21 rows, ~400K distinct strings of 1-24 bytes (partitioned strategy chosen by the
    sketch), device-resident input."""
    rng = np.random.default_rng(77)
    n = 1 << 21
    keys = _strings(rng, n, 600_000, max_len=24)
    km = rng.random(n) < 0.01
    _check([keys], [V], [km], *_values(rng, n), batch_sizes=(4096,), device_input=True)


def _expected_min_max(keys, kmask, vals, vmask):
    want = {}
    for k, km, v, vm in zip(keys.tolist(), kmask.tolist(), vals, vmask.tolist()):
        g = (None if km else int(k),)
        lo, hi, c = want.get(g, (None, None, 0))
        if not vm:
            b = bytes(v)
            lo = b if lo is None or b < lo else lo
            hi = b if hi is None or b > hi else hi
            c += 1
        want[g] = (lo, hi, c)
    return want


@pytest.mark.parametrize("strategy", [omg.AGG_STRATEGY_AUTO, omg.AGG_STRATEGY_GLOBAL, omg.AGG_STRATEGY_SMEM,
                                      omg.AGG_STRATEGY_PARTITIONED])
@pytest.mark.parametrize("flush_rows", [0, 9000])
def test_varchar_min_max_match_python(strategy, flush_rows):
    """MIN and MAX of a VARCHAR column (with NULLs, empty strings, shared prefixes and bytes above
    0x7f) per int64 group, against byte-wise comparison; small flushes make later batch sets
    compare new strings with ids stored by earlier ones."""
    rng = np.random.default_rng(31 + strategy + flush_rows)
    n = 150_000
    pool = [bytes(rng.integers(0, 256, l, dtype=np.uint8)) for l in rng.integers(0, 12, 3000)]
    pool += [b"", b"a", b"ab", b"abc", b"\xff", b"\xff\x00"]
    vals = np.array([pool[i] for i in rng.integers(0, len(pool), n)], dtype=object)
    vm = rng.random(n) < 0.05
    keys = rng.integers(0, 700, n).astype(np.int64)
    km = rng.random(n) < 0.01
    if flush_rows:
        omg.lib().omg_debug_set_agg_flush_rows(flush_rows)
    try:
        cols, _ = run_agg([0], [L], [[1], [1], [1]], [[V], [V], [V]], [[V], [V], [L]], [MIN, MAX, CNT],
                          [keys, vals], [L, V], nulls=[km, vm], batch_sizes=(4096, 1003), strategy=strategy)
    finally:
        omg.lib().omg_debug_set_agg_flush_rows(0)
    assert _str_rows(cols, 1) == _expected_min_max(keys, km, vals, vm)
