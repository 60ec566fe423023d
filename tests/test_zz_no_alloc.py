"""The allocation-free aggregation entry point (omg_hashagg_run_noalloc) through the C ABI.

It exists for callers that cannot let the library allocate device memory: an engine that keeps
all device memory in its own pre-reserved pool, or code running where allocation calls are not
permitted.  Its scratch is a fixed device array inside the library, shared by every call.  These
tests check its output against the operator API (the existing entry point) and against the
oracle on the same inputs, for two calls in a row (the second call must not see the first
call's leftovers), with and without null bitmaps, and its two rejections: a size beyond the
scratch (before any device work) and an input with more groups than max_groups (found on the
device).  They sit in a file of their own that pytest collects last, and pass alone in a fresh
process as well.
"""
import ctypes as C

import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import DOUBLE_TOL, assert_agg_equal, exact_by_key, run_agg

pytestmark = pytest.mark.gpu

L, D = omg.LongType(), omg.DoubleType()
SUM, CNT, AVG, MAX, MIN = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                           omg.OMNI_AGGREGATION_TYPE_AVG, omg.OMNI_AGGREGATION_TYPE_MAX,
                           omg.OMNI_AGGREGATION_TYPE_MIN)
SPEC = dict(group_cols=[0], group_types=[L], aggs_cols=[[1], [1], [1], [1], [2], [2]],
            agg_in_types=[[L], [L], [L], [L], [D], [D]], agg_out_types=[[L], [L], [L], [L], [D], [D]],
            funcs=[SUM, CNT, MIN, MAX, SUM, AVG])
OUT_TYPES = [L, L, L, L, L, D, D]


def _data(seed, n=150_000, groups=3000):
    rng = np.random.default_rng(seed)
    uniq = rng.integers(-2**62, 2**62, groups, dtype=np.int64)
    key = uniq[rng.integers(0, groups, n)]
    v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    v2 = rng.random(n)
    m1 = rng.random(n) < 0.02
    km = rng.random(n) < 0.01
    return key, v1, v2, km, m1


def _rows(cols):
    """{key (None for NULL): (values or None for NULL, ...)} from [(values, mask)] columns."""
    out = {}
    for i in range(len(cols[0][0])):
        k = None if cols[0][1][i] else int(cols[0][0][i])
        out[k] = tuple(None if m[i] else v[i] for v, m in cols[1:])
    return out


def _run_noalloc(fac, key, v1, v2, km, m1, max_groups, out_rows=None, num_groups=None):
    """One omg_hashagg_run_noalloc call over device copies of the columns.  km / m1 None: the
    call gets a NULL null-bitmap array (no column has nulls).  Returns (output columns, groups);
    `num_groups` (a c_int64) receives the group count when given."""
    L_ = omg.lib()
    host = omg.make_batch([L, L, D], [key, v1, v2], [km, m1, None])
    dev = omg.batch_to_device(host)
    omg.free_batch(host)
    outs = []
    try:
        cols = (C.c_void_p * 3)(*[L_.omg_vec_values(L_.omg_batch_get(dev, i)) for i in range(3)])
        if km is None and m1 is None:
            nulls = None
        else:
            nulls = (C.c_void_p * 3)(*[L_.omg_vec_nulls(L_.omg_batch_get(dev, i)) if L_.omg_vec_has_null(
                L_.omg_batch_get(dev, i)) else None for i in range(3)])
        # The caller allocates the outputs (here through the library's device vectors).
        for t in OUT_TYPES:
            v = C.c_void_p()
            omg._capi.check(L_.omg_vec_new_device(t.id, 0, max_groups if out_rows is None else out_rows,
                                                  C.byref(v)))
            outs.append(v.value)
        ov = (C.c_void_p * len(outs))(*[L_.omg_vec_values(v) for v in outs])
        on = (C.c_void_p * len(outs))(*[L_.omg_vec_nulls(v) for v in outs])
        ng = C.c_int64(-1) if num_groups is None else num_groups
        rc = L_.omg_hashagg_run_noalloc(fac.handle, cols, nulls, 3, len(key), ov, on, len(outs), max_groups,
                                        C.byref(ng), None)
        omg._capi.check(rc)
        # Read the first ng rows back through a host batch.
        b = C.c_void_p()
        omg._capi.check(L_.omg_batch_new(ng.value, C.byref(b)))
        for v in outs:
            w = C.c_void_p()
            omg._capi.check(L_.omg_vec_wrap_device(L_.omg_vec_type(v), 0, ng.value, L_.omg_vec_values(v),
                                                   L_.omg_vec_nulls(v), C.byref(w)))
            omg._capi.check(L_.omg_batch_append(b.value, w.value))
        hb = omg.batch_to_host(b.value)
        omg.free_batch(b.value)
        res = omg.batch_to_numpy(hb)
        omg.free_batch(hb)
        return res, ng.value
    finally:
        for v in outs:
            L_.omg_vec_free(v)
        omg.free_batch(dev)


def _assert_same(a, b):
    ra, rb = _rows(a), _rows(b)
    assert ra.keys() == rb.keys()
    for k in ra:
        for j, (x, y) in enumerate(zip(ra[k], rb[k])):
            if x is None or y is None:
                assert x is None and y is None, (k, j)
            elif j >= 4:  # double SUM / AVG: the tolerance the double tests use
                assert abs(float(x) - float(y)) <= DOUBLE_TOL * max(abs(float(y)), 1.0), (k, j, x, y)
            else:
                assert int(x) == int(y), (k, j, x, y)


def _assert_matches_oracle(got, key, km, v1, m1, v2):
    ora = oracle.hashagg(
        [key], [oracle.T_LONG], [km],
        [dict(func=oracle.F_SUM, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_COUNT_COL, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MIN, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_MAX, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m1),
         dict(func=oracle.F_SUM, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE),
         dict(func=oracle.F_AVG, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE)])
    ex_sum = exact_by_key([key], [km], v2, None)
    ex_avg = exact_by_key([key], [km], v2, None, divide_by_count=True)
    assert_agg_equal(got, ora, 1, double_aggs=(4, 5), exact={4: ex_sum, 5: ex_avg})


def test_noalloc_matches_oracle_twice_with_and_without_nulls(gpu):
    """Two calls in a row on one factory: the first with NULL keys and values, the second with
    no null bitmaps at all (d_nulls = NULL) and fewer groups, each against the oracle."""
    fac = omg.HashAggregationOperatorFactory([0], [L], SPEC["aggs_cols"], SPEC["agg_in_types"],
                                             SPEC["agg_out_types"], SPEC["funcs"])
    try:
        key, v1, v2, km, m1 = _data(11, groups=2500)
        got, ng = _run_noalloc(fac, key, v1, v2, km, m1, max_groups=4096)
        _assert_matches_oracle(got, key, km, v1, m1, v2)
        key, v1, v2, _, _ = _data(12, groups=300)
        got, ng = _run_noalloc(fac, key, v1, v2, None, None, max_groups=4096)
        assert ng == len(np.unique(key))
        _assert_matches_oracle(got, key, None, v1, None, v2)
    finally:
        fac.close()


def test_noalloc_rejects_more_groups_than_max_groups(gpu):
    """5,000 distinct keys with max_groups = 1,024: the table (2,048 slots) overflows on the
    device; the call returns OMG_ERR_INVALID_ARG and leaves num_groups untouched.  A call that
    follows on the same factory still agrees with the oracle."""
    fac = omg.HashAggregationOperatorFactory([0], [L], SPEC["aggs_cols"], SPEC["agg_in_types"],
                                             SPEC["agg_out_types"], SPEC["funcs"])
    try:
        key = np.arange(5000, dtype=np.int64) * 7919
        rng = np.random.default_rng(5)
        v1 = rng.integers(-100, 100, len(key), dtype=np.int64)
        v2 = rng.random(len(key))
        ng = C.c_int64(-12345)
        with pytest.raises(omg.OmgError) as e:
            _run_noalloc(fac, key, v1, v2, None, None, max_groups=1024, num_groups=ng)
        assert e.value.status == -1 and "max_groups" in e.value.message  # OMG_ERR_INVALID_ARG
        assert ng.value == -12345
        key, v1, v2, km, m1 = _data(13, n=40_000, groups=900)
        got, _ = _run_noalloc(fac, key, v1, v2, km, m1, max_groups=1024)
        _assert_matches_oracle(got, key, km, v1, m1, v2)
    finally:
        fac.close()


def test_noalloc_matches_operator_api_twice(gpu):
    fac = omg.HashAggregationOperatorFactory([0], [L], SPEC["aggs_cols"], SPEC["agg_in_types"],
                                             SPEC["agg_out_types"], SPEC["funcs"])
    try:
        for seed, groups in ((1, 3000), (2, 700)):
            key, v1, v2, km, m1 = _data(seed, groups=groups)
            expected, _ = run_agg(**SPEC, columns=[key, v1, v2], types=[L, L, D], nulls=[km, m1, None])
            got, ng = _run_noalloc(fac, key, v1, v2, km, m1, max_groups=4096)
            assert ng == len(expected[0][0])
            _assert_same(got, expected)
    finally:
        fac.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    fac = omg.HashAggregationOperatorFactory([0], [L], SPEC["aggs_cols"], SPEC["agg_in_types"],
                                             SPEC["agg_out_types"], SPEC["funcs"])
    try:
        key, v1, v2, km, m1 = _data(3, n=1000, groups=10)
        with pytest.raises(omg.OmgError) as e:
            # The call is rejected before it touches the (here deliberately small) outputs.
            _run_noalloc(fac, key, v1, v2, km, m1, max_groups=50_000_000, out_rows=16)
        assert e.value.status == -1 and "scratch" in e.value.message
    finally:
        fac.close()
