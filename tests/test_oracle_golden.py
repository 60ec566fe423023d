"""Pins the CPU oracle to the reference's own known-answer tests (tests/golden/*.json, transcribed
from core/test/operator/{aggregation,join}_test.cpp) and checks it against brute-force numpy
restatements on random inputs.  CPU only."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import oracle_join_rows, row_key

G = Path(__file__).parent / "golden"
TYPES = {"LONG": oracle.T_LONG, "DOUBLE": oracle.T_DOUBLE, "DECIMAL64": oracle.T_DEC64,
         "DECIMAL128": oracle.T_DEC128, "INT": oracle.T_INT}
FUNCS = {"SUM": oracle.F_SUM, "AVG": oracle.F_AVG, "COUNT_COLUMN": oracle.F_COUNT_COL, "MIN": oracle.F_MIN,
         "MAX": oracle.F_MAX, "COUNT_ALL": oracle.F_COUNT_ALL}


def _col(values, t):
    if t == "DECIMAL128":
        return np.array([[v & (2**64 - 1), (v >> 64) & (2**64 - 1)] for v in values], dtype=np.uint64)
    if t == "DOUBLE":
        return np.array(values, dtype=np.float64)
    return np.array(values, dtype=np.int64)


def _dec128(pair):
    v = int(pair[0]) | (int(pair[1]) << 64)
    return v - (1 << 128) if v >= 1 << 127 else v


AGG = json.loads((G / "agg_kats.json").read_text())
JOIN = json.loads((G / "join_kats.json").read_text())


@pytest.mark.parametrize("name", sorted(AGG["single"]))
@pytest.mark.parametrize("as_null", [False, True])
def test_oracle_single_aggregate_kats(name, as_null):
    k = AGG["single"][name]
    n = len(k["values"])
    key = np.zeros(n, dtype=np.int64)
    col = _col(k["values"], k["in_type"])
    nulls = None if k["nulls"] is None else np.array(k["nulls"], dtype=bool)
    agg = dict(func=FUNCS[k["func"]], col=col, in_type=TYPES[k["in_type"]], out_type=TYPES[k["out_type"]],
               nulls=nulls)
    policy = 0 if k["policy"] == "spark" else 1
    if k["expected"] == "overflow":
        if as_null:
            _, _, vals, vnulls = oracle.hashagg([key], [oracle.T_LONG], [None], [agg], policy, True)
            assert vnulls[0][0]
        else:
            with pytest.raises(OverflowError):
                oracle.hashagg([key], [oracle.T_LONG], [None], [agg], policy, False)
        return
    _, _, vals, vnulls = oracle.hashagg([key], [oracle.T_LONG], [None], [agg], policy, as_null)
    if k["expected"] is None:
        assert vnulls[0][0]
        return
    assert not vnulls[0][0]
    got = vals[0][0]
    if k["out_type"] == "DECIMAL128":
        assert _dec128(got) == k["expected"]
    elif k["out_type"] == "DOUBLE":
        assert float(got) == k["expected"]  # the reference's naive fold, reproduced bit for bit
    else:
        assert int(got) == k["expected"]


def test_oracle_verify_null_correctness():
    k = AGG["multi"]["verify_null_correctness"]
    key = np.array(k["key"], dtype=np.int64)
    aggs = []
    for f, c, m, t in zip(k["funcs"], k["columns"], k["nulls"], k["out_types"]):
        aggs.append(dict(func=FUNCS[f], col=np.array(c, dtype=np.int64), in_type=oracle.T_LONG,
                         out_type=TYPES[t], nulls=np.array(m, dtype=bool)))
    keys, knulls, vals, vnulls = oracle.hashagg([key], [oracle.T_LONG], [None], aggs)
    row = [int(keys[0][0])] + [float(v[0]) if t == "DOUBLE" else int(v[0]) for v, t in zip(vals, k["out_types"])]
    assert row == k["expected"][0]
    assert not any(m[0] for m in vnulls)


@pytest.mark.parametrize("name", sorted(JOIN))
def test_oracle_join_kats(name):
    k = JOIN[name]
    b = [np.array(c, dtype=np.int64) for c in k["build"]]
    p = [np.array(c, dtype=np.int64) for c in k["probe"]]
    pi, bi = oracle.join_inner(b[k["build_hash_col"]], None, p[k["probe_hash_col"]], None)
    rows = sorted(tuple(int(p[c][i]) for c in k["probe_output_cols"]) + tuple(int(b[c][j]) for c in k["build_output_cols"])
                  for i, j in zip(pi, bi))
    assert rows == sorted(tuple(r) for r in k["expected_rows"])


JOIN_TYPED = json.loads((G / "join_type_kats.json").read_text())


@pytest.mark.parametrize("name", sorted(JOIN_TYPED))
def test_oracle_join_type_kats(name):
    k = JOIN_TYPED[name]
    rows, outer = oracle_join_rows(k)
    assert sorted(map(row_key, rows)) == sorted(map(row_key, k["expected_rows"]))
    if k["outer_rows"] is not None:  # None: the reference test does not read the outer rows
        assert sorted(map(row_key, outer)) == sorted(map(row_key, k["outer_rows"]))


def test_oracle_join_kinds_match_bruteforce():
    rng = np.random.default_rng(5)
    bk = rng.integers(-20, 20, 200).astype(np.int64)
    bn = rng.random(200) < 0.1
    pk = rng.integers(-25, 25, 300).astype(np.int64)
    pn = rng.random(300) < 0.1
    match = [[j for j in range(200) if not pn[i] and not bn[j] and bk[j] == pk[i]] for i in range(300)]
    hit = set(j for m in match for j in m)
    unhit = [(-1, j) for j in range(200) if j not in hit]
    pairs = [(i, j) for i in range(300) for j in match[i]]
    lone = [(i, -1) for i in range(300) if not match[i]]
    expect = {"inner": pairs, "probe_outer": pairs + lone, "build_outer": pairs + unhit,
              "full": pairs + lone + unhit, "semi": [(i, -1) for i in range(300) if match[i]],
              "anti": lone, "existence": [(i, 1 if match[i] else 0) for i in range(300)]}
    for kind, exp in expect.items():
        pi, bi = oracle.join(kind, bk, bn, pk, pn)
        assert sorted(zip(pi.tolist(), bi.tolist())) == sorted(exp), kind


def test_oracle_join_matches_bruteforce():
    rng = np.random.default_rng(3)
    for trial in range(5):
        bk = rng.integers(-50, 50, 300).astype(np.int64)
        bn = rng.random(300) < 0.1
        pk = rng.integers(-60, 60, 500).astype(np.int64)
        pn = rng.random(500) < 0.1
        pi, bi = oracle.join_inner(bk, bn, pk, pn)
        got = sorted(zip(pi.tolist(), bi.tolist()))
        exp = sorted((i, j) for i in range(500) if not pn[i] for j in range(300) if not bn[j] and bk[j] == pk[i])
        assert got == exp


def test_oracle_sparse_keys_hash_mode_matches_bruteforce():
    rng = np.random.default_rng(4)
    bk = rng.integers(-2**62, 2**62, 400, dtype=np.int64)
    bk[:50] = bk[50:100]
    pk = np.concatenate([bk[rng.integers(0, 400, 300)], rng.integers(-2**62, 2**62, 200, dtype=np.int64)])
    pi, bi = oracle.join_inner(bk, None, pk, None)
    got = sorted(zip(pi.tolist(), bi.tolist()))
    idx = {}
    for j, k in enumerate(bk.tolist()):
        idx.setdefault(k, []).append(j)
    exp = sorted((i, j) for i, k in enumerate(pk.tolist()) for j in idx.get(k, []))
    assert got == exp


def test_oracle_agg_matches_numpy():
    rng = np.random.default_rng(5)
    n = 20000
    key = rng.integers(0, 97, n).astype(np.int64)
    v = rng.integers(-10**12, 10**12, n, dtype=np.int64)
    m = rng.random(n) < 0.05
    aggs = [dict(func=f, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG, nulls=m)
            for f in (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_MIN, oracle.F_MAX)]
    aggs.append(dict(func=oracle.F_COUNT_ALL, col=None, out_type=oracle.T_LONG))
    keys, _, vals, vn = oracle.hashagg([key], [oracle.T_LONG], [None], aggs)
    for i, k in enumerate(keys[0]):
        sel = (key == k) & ~m
        assert int(vals[0][i]) == int(v[sel].sum())
        assert int(vals[1][i]) == int(sel.sum())
        assert int(vals[2][i]) == int(v[sel].min())
        assert int(vals[3][i]) == int(v[sel].max())
        assert int(vals[4][i]) == int((key == k).sum())


def test_oracle_generic_sticky_overflow_is_order_dependent():
    big = 2**62
    key = np.array([0, 0, 0, 0, 1, 1, 1, 1], dtype=np.int64)
    v = np.array([big, big, -big, -big, big, -big, big, -big], dtype=np.int64)
    agg = dict(func=oracle.F_SUM, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)
    keys, _, vals, vn = oracle.hashagg([key], [oracle.T_LONG], [None], [agg], policy=1, overflow_as_null=True)
    res = {int(k): (bool(vn[0][i]), int(vals[0][i])) for i, k in enumerate(keys[0])}
    assert res[0][0] is True          # 2^62 + 2^62 overflows int64 on the second row
    assert res[1] == (False, 0)       # interleaved order never leaves the range
    _, _, vals, vn = oracle.hashagg([key], [oracle.T_LONG], [None], [agg], policy=0)
    assert not vn[0].any()            # Spark policy wraps: both groups sum to 0
    assert all(int(x) == 0 for x in vals[0])


def test_filtered_join_restatement_reduces_to_the_plain_join():
    """oracle.join_filtered with an always-true filter equals oracle.join for every kind, and
    an always-false filter leaves no match (random keys with NULLs and duplicate build keys)."""
    rng = np.random.default_rng(3)
    bk = rng.integers(0, 50, 300).astype(np.int64)
    bn = rng.random(300) < 0.05
    pk = rng.integers(0, 80, 500).astype(np.int64)
    pn = rng.random(500) < 0.05
    for kind in oracle.JOIN_KINDS:
        a = oracle.join(kind, bk, bn, pk, pn)
        b = oracle.join_filtered(kind, bk, bn, pk, pn, lambda p, q: np.ones(len(p), bool))
        assert sorted(zip(*[x.tolist() for x in a])) == sorted(zip(*[x.tolist() for x in b]))
        none = oracle.join_filtered(kind, bk, bn, pk, pn, lambda p, q: np.zeros(len(p), bool))
        if kind in ("inner", "semi"):
            assert len(none[0]) == 0
        if kind == "existence":
            assert not none[1].any()


ARRAY_MAP = AGG["array_map"]
KEY_NP = {"SHORT": (np.int16, oracle.T_SHORT), "INT": (np.int32, oracle.T_INT), "DATE32": (np.int32, oracle.T_DATE32),
          "LONG": (np.int64, oracle.T_LONG), "TIMESTAMP": (np.int64, oracle.T_LONG),
          "DECIMAL64": (np.int64, oracle.T_DEC64)}


def array_map_inputs(k):
    """Concatenated key column, key NULLs, five aggregate columns (ones) and their NULLs."""
    dt = KEY_NP[k["key_type"]][0]
    keys, knull, anulls = [], [], [[] for _ in range(5)]
    for b in k["batches"]:
        keys += b["keys"]
        knull += [r in b["key_nulls"] for r in range(21)]
        for c in range(5):
            anulls[c] += [r in b["agg_nulls"][c] for r in range(21)]
    return (np.array(keys, dtype=dt), np.array(knull, dtype=bool), np.ones(len(keys), dtype=np.int64),
            [np.array(m, dtype=bool) for m in anulls])


def array_map_rows(keys, knulls, vals, vnulls, n_aggs):
    rows = []
    for i in range(len(keys)):
        r = [None if knulls[i] else int(keys[i])]
        for j in range(n_aggs):
            v = vals[j][i]
            r.append(None if vnulls[j][i] else (float(v) if j == 1 else int(v)))
        rows.append(r)
    return sorted(rows, key=lambda r: (r[0] is None, r[0] if r[0] is not None else 0))


@pytest.mark.parametrize("name", sorted(ARRAY_MAP))
def test_oracle_array_map_kats(name):
    k = ARRAY_MAP[name]
    key, knull, ones, anulls = array_map_inputs(k)
    funcs = [] if k.get("no_aggs") else ["SUM", "AVG", "COUNT_COLUMN", "MIN", "MAX"]
    outs = [oracle.T_DOUBLE if f == "AVG" else oracle.T_LONG for f in funcs]
    aggs = [dict(func=FUNCS[f], col=ones, in_type=oracle.T_LONG, out_type=o, nulls=anulls[j])
            for j, (f, o) in enumerate(zip(funcs, outs))]
    keys, knulls, vals, vnulls = oracle.hashagg([key], [KEY_NP[k["key_type"]][1]], [knull], aggs)
    got = array_map_rows(keys[0], knulls[0], vals, vnulls, len(funcs))
    want = sorted(k["expected"], key=lambda r: (r[0] is None, r[0] if r[0] is not None else 0))
    assert got == want


SUBSTR = json.loads((Path(__file__).parent / "golden" / "substr_kats.json").read_text(encoding="utf-8"))


@pytest.mark.parametrize("name", sorted(SUBSTR))
def test_oracle_substr_kats(name):
    """oracle.substr against the reference's substr function tests (UTF-8 code points, the four
    start-index policies)."""
    for c in SUBSTR[name]["cases"]:
        got = oracle.substr(c["string"].encode(), c["start"], c["length"], c["negative"], c["zero"])
        assert got == c["expected"].encode(), c


def test_oracle_str_compare_is_unsigned_bytes_then_length():
    assert oracle.str_compare(b"abc", b"abd") == -1
    assert oracle.str_compare(b"ab", b"abc") == -1
    assert oracle.str_compare(b"\xc3\xa9", b"z") == 1  # bytes above 0x7f compare as unsigned
    assert oracle.str_compare(b"", b"") == 0


# core/test/codegen/function_test.cpp:2623-2800 (InStr, StartsWithStr, EndsWithStr, LengthStr,
# LengthStrZh, CharLengthStr, LengthChar, CharLengthChar) and :3741-3797 (ContainsStr): the
# non-NULL calls; a NULL argument makes the expression NULL (the INPUT_DATA registrations).
STRING_FN_KATS = [
    ("instr", ["abc", "abcd"], 0), ("instr", ["abc", "bd"], 0), ("instr", ["abc", "bc"], 2),
    ("instr", ["", "ab"], 0), ("instr", ["abc", ""], 1), ("instr", ["", ""], 1),
    ("instr", ["一丁丂七丄丅丆万丈三上下丌不与丏", "万丈"], 8), ("instr", ["壹貳叁肆伍", "叁肆"], 3),
    ("StartsWith", ["abc", "abcd"], 0), ("StartsWith", ["abc", "bd"], 0), ("StartsWith", ["abc", "ab"], 1),
    ("StartsWith", ["", "ab"], 0), ("StartsWith", ["abc", ""], 1), ("StartsWith", ["", ""], 1),
    ("EndsWith", ["abc", "abcd"], 0), ("EndsWith", ["abc", "bd"], 0), ("EndsWith", ["abc", "bc"], 1),
    ("EndsWith", ["", "ab"], 0), ("EndsWith", ["abc", ""], 1), ("EndsWith", ["", ""], 1),
    ("length", ["abcd"], 4), ("length", ["时欧基乌斯侧后解 hello! 回复哦黑色的and magic粉色的圣诞袜"], 37),
    ("char_length", ["m"], 1),
    ("Contains", ["", "abc"], 0), ("Contains", ["abc", "abd"], 0), ("Contains", ["abcd", "abd"], 0),
    ("Contains", ["abcd", "acd"], 0),
]


@pytest.mark.parametrize("name,args,expected", STRING_FN_KATS)
def test_oracle_string_function_kats(name, args, expected):
    assert oracle.string_function(name, [a.encode() for a in args]) == expected


def test_oracle_string_function_nulls_and_extremes():
    assert oracle.string_function("instr", [None, b"a"]) is None
    assert oracle.string_function("length", [b"abcd"], char_width=10) == 10  # LengthChar: the width
    assert oracle.string_function("Greatest", [b"ab", b"abc"]) == b"abc"
    assert oracle.string_function("Least", [b"ab", b"abc"]) == b"ab"
    assert oracle.string_function("Greatest", [None, b"x"]) == b"x"
    assert oracle.string_function("Least", [None, None]) is None
