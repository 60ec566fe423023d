"""Parity at the full size of the two headline configurations, through the C ABI, against the
oracle: the uniform aggregation (2^22 rows, 10,000 groups; every group) and the inner-join
probe (2^20 build rows, 2^26 probe rows; the row multiset by a 128-bit fingerprint and the row
count).  The inputs are the bench's own seeded data.  Also pins the device fingerprint kernel
to the oracle's restatement of it, which the full-size join check relies on."""
import numpy as np
import pytest

import bench
import omnioperator_gb300 as omg
import oracle

pytestmark = pytest.mark.gpu

L, I, D, S = omg.LongType(), omg.IntType(), omg.DoubleType(), omg.ShortType()
D128 = omg.Decimal128Type(38, 2)


def test_device_fingerprint_equals_oracle_fingerprint(gpu):
    rng = np.random.default_rng(21)
    n = 70_000
    cols = [rng.integers(-2**63, 2**63 - 1, n, dtype=np.int64), rng.integers(-2**31, 2**31, n).astype(np.int32),
            rng.integers(-2**15, 2**15, n).astype(np.int16), rng.integers(0, 2**64 - 1, (n, 2), dtype=np.uint64)]
    nulls = [None, rng.random(n) < 0.1, rng.random(n) < 0.5, rng.random(n) < 0.05]
    types = [L, I, S, D128]
    batches = [omg.make_batch(types, [c[s:s + 5000] for c in cols],
                              [None if m is None else m[s:s + 5000] for m in nulls]) for s in range(0, n, 5000)]
    try:
        host_fp = omg.batches_fingerprint(batches)
        dev = [omg.batch_to_device(b) for b in batches]
        dev_fp = omg.batches_fingerprint(dev)
        omg.free_batches(dev)
    finally:
        omg.free_batches(batches)
    ref = oracle.fingerprint_cols(cols, nulls)
    assert tuple(host_fp) == ref and tuple(dev_fp) == ref


def test_uniform_aggregation_full_size(gpu):
    """All 2^22 rows of the uniform-key workload, all 10,000 groups against the oracle."""
    key, v1, v2 = bench.agg_data_numpy(2)
    fac = omg.HashAggregationOperatorFactory(
        [0], [L], [[1], [1], [1], [1], [2], [2]], [[L], [L], [L], [L], [D], [D]], [[L], [L], [L], [L], [D], [D]],
        [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN, omg.OMNI_AGGREGATION_TYPE_MIN,
         omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_AVG])
    op = fac.create_operator()
    try:
        for s in range(0, len(key), bench.BATCH):
            op.add_input(omg.make_batch([L, L, D], [key[s:s + bench.BATCH], v1[s:s + bench.BATCH],
                                                    v2[s:s + bench.BATCH]]))
        cols = bench.host_columns(omg, op.drain())
    finally:
        op.delete()
        fac.close()
    res = bench.check_agg_uniform(key, v1, v2, cols)
    assert res["groups"] == bench.AGG_GROUPS
    assert res["oracle_match"], res


def test_join_probe_full_size(gpu):
    """All 2^26 probe rows of the headline join (device-resident input, device output): row
    count and row-multiset fingerprint against the oracle's join."""
    bkey, p1, p2, pkey, pnull = bench.join_data_numpy(1)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I, I], [0])
    bop = bf.create_operator()
    pf = pop = None
    try:
        bop.add_input(omg.make_batch([L, I, I], [bkey, p1, p2]))
        bop.get_output()
        pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf)
        pop = pf.create_operator()
        pop.set_device_output(True)
        fp = [0, 0, 0]
        for s in range(0, len(pkey), 1 << 24):
            h = omg.make_batch([L], [pkey[s:s + (1 << 24)]], [pnull[s:s + (1 << 24)]])
            d = omg.batch_to_device(h)
            omg.free_batch(h)
            pop.add_input(d)
            outs, _ = pop.get_outputs(1 << 16)
            f = omg.batches_fingerprint(outs)
            fp = [(a + b) & ((1 << 64) - 1) for a, b in zip(fp, f)]
            omg.free_batches(outs)
    finally:
        if pop:
            pop.delete()
        bop.delete()
        if pf:
            pf.close()
        bf.close()
    res = bench.check_join_fingerprint(fp, bkey, [p1, p2], pkey, pnull)
    assert res["rows"] == int((~pnull & (pkey < bench.N_BUILD)).sum())
    assert res["oracle_match"], res
