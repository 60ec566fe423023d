"""The reference's known-answer tests (tests/golden/agg_kats.json) through the GPU operators.
Integer/decimal results must equal the reference's expected values exactly; double results
within 1e-12 relative of them (the reference's own value is a naive fold, the GPU's a
compensated sum)."""
import json
from pathlib import Path

import numpy as np
import pytest

import omnioperator_gb300 as omg
from helpers import run_agg

pytestmark = pytest.mark.gpu

AGG = json.loads((Path(__file__).parent / "golden" / "agg_kats.json").read_text())
FUNCS = {"SUM": omg.OMNI_AGGREGATION_TYPE_SUM, "AVG": omg.OMNI_AGGREGATION_TYPE_AVG,
         "COUNT_COLUMN": omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN, "MIN": omg.OMNI_AGGREGATION_TYPE_MIN,
         "MAX": omg.OMNI_AGGREGATION_TYPE_MAX}


def _type(name, scale=0):
    return {"LONG": omg.LongType(), "DOUBLE": omg.DoubleType(), "DECIMAL64": omg.Decimal64Type(18, scale),
            "DECIMAL128": omg.Decimal128Type(38, scale)}[name]


def _col(values, t):
    if t == "DECIMAL128":
        return np.array([[v & (2**64 - 1), (v >> 64) & (2**64 - 1)] for v in values], dtype=np.uint64)
    return np.array(values, dtype=np.float64 if t == "DOUBLE" else np.int64)


@pytest.mark.parametrize("name", sorted(AGG["single"]))
@pytest.mark.parametrize("as_null", [False, True])
def test_single_aggregate_kats_on_gpu(gpu, name, as_null):
    k = AGG["single"][name]
    n = len(k["values"])
    key = np.zeros(n, dtype=np.int64)
    tin = _type(k["in_type"], k.get("scale", 0))
    tout = _type(k["out_type"], k.get("scale", 0))
    col = _col(k["values"], k["in_type"])
    nulls = [None, None if k["nulls"] is None else np.array(k["nulls"], dtype=bool)]
    omg.set_policy(omg.POLICY_SPARK if k["policy"] == "spark" else omg.POLICY_GENERIC)
    try:
        args = ([0], [omg.LongType()], [[1]], [[tin]], [[tout]], [FUNCS[k["func"]]], [key, col],
                [omg.LongType(), tin])
        if k["expected"] == "overflow" and not as_null:
            with pytest.raises(omg.OmgError) as e:
                run_agg(*args, nulls=nulls, overflow_as_null=False)
            assert e.value.status == -5
            return
        cols, _ = run_agg(*args, nulls=nulls, overflow_as_null=as_null)
    finally:
        omg.set_policy(omg.POLICY_SPARK)
    vals, mask = cols[1]
    if k["expected"] in (None, "overflow"):
        assert mask[0]
        return
    assert not mask[0]
    if k["out_type"] == "DECIMAL128":
        v = int(vals[0][0]) | (int(vals[0][1]) << 64)
        v = v - (1 << 128) if v >= 1 << 127 else v
        assert v == k["expected"]
    elif k["out_type"] == "DOUBLE":
        assert abs(float(vals[0]) - k["expected"]) <= 1e-12 * abs(k["expected"])
    else:
        assert int(vals[0]) == k["expected"]


def test_verify_null_correctness_on_gpu(gpu):
    k = AGG["multi"]["verify_null_correctness"]
    L, D = omg.LongType(), omg.DoubleType()
    key = np.array(k["key"], dtype=np.int64)
    cols_in = [np.array(c, dtype=np.int64) for c in k["columns"]]
    outs = [[D] if t == "DOUBLE" else [L] for t in k["out_types"]]
    cols, _ = run_agg([0], [L], [[1], [2], [3], [4], [5]], [[L]] * 5, outs, [FUNCS[f] for f in k["funcs"]],
                      [key] + cols_in, [L] * 6, nulls=[None] + [np.array(m, bool) for m in k["nulls"]])
    row = [int(cols[0][0][0])] + [float(c[0][0]) if t == "DOUBLE" else int(c[0][0])
                                  for c, t in zip(cols[1:], k["out_types"])]
    assert row == k["expected"][0]


ARRAY_MAP = AGG["array_map"]
KEY_TYPES = {"SHORT": (np.int16, omg.ShortType()), "INT": (np.int32, omg.IntType()),
             "DATE32": (np.int32, omg.DataType(omg.OMNI_DATE32)), "LONG": (np.int64, omg.LongType()),
             "TIMESTAMP": (np.int64, omg.DataType(omg.OMNI_TIMESTAMP)), "DECIMAL64": (np.int64, omg.Decimal64Type(18, 0))}


@pytest.mark.parametrize("name", sorted(ARRAY_MAP))
def test_array_map_kats_on_gpu(gpu, name):
    """The reference's ArrayMap tests (aggregation_test.cpp:632-1190): NULL keys, NULL values,
    a key far outside the first batch's range and the key type's min / max, two batches."""
    k = ARRAY_MAP[name]
    dt, kt = KEY_TYPES[k["key_type"]]
    L, D = omg.LongType(), omg.DoubleType()
    keys, knull, anulls = [], [], [[] for _ in range(5)]
    for b in k["batches"]:
        keys += b["keys"]
        knull += [r in b["key_nulls"] for r in range(21)]
        for c in range(5):
            anulls[c] += [r in b["agg_nulls"][c] for r in range(21)]
    key = np.array(keys, dtype=dt)
    ones = np.ones(len(keys), dtype=np.int64)
    no_aggs = k.get("no_aggs", False)
    funcs = [] if no_aggs else [FUNCS[f] for f in ("SUM", "AVG", "COUNT_COLUMN", "MIN", "MAX")]
    n_agg = len(funcs)
    cols, _ = run_agg([0], [kt], [[1 + j] for j in range(n_agg)], [[L]] * n_agg,
                      [[D] if j == 1 else [L] for j in range(n_agg)], funcs, [key] + [ones] * n_agg,
                      [kt] + [L] * n_agg, nulls=[np.array(knull)] + [np.array(m) for m in anulls[:n_agg]],
                      batch_sizes=(21,))
    rows = []
    for i in range(len(cols[0][0])):
        r = [None if cols[0][1][i] else int(cols[0][0][i])]
        for j in range(n_agg):
            v, m = cols[1 + j]
            r.append(None if m[i] else (float(v[i]) if j == 1 else int(v[i])))
        rows.append(r)
    order = lambda r: (r[0] is None, r[0] if r[0] is not None else 0)  # noqa: E731
    assert sorted(rows, key=order) == sorted(k["expected"], key=order)
