"""Join filters over strings and conditionals on the GPU: VARCHAR/CHAR columns and literals of both
sides compared byte-wise (unsigned, a proper prefix first), substr over UTF-8 code points under
the four start-index policies, and IF / CASE / COALESCE / IN / BETWEEN with the reference's NULL
rules (codegen/expression_codegen.cpp:352-760) (lookup_join.cpp:175-187,1440-1466; codegen/functions/stringfunctions.h:
215-318).  Known answers: the reference's CHAR-filter join tests (join_test.cpp:1796-2150) with
their expected rows, and its substr function tests (function_test.cpp:2030-2506, the vectors in
tests/golden/substr_kats.json) evaluated by the probe kernel.  Random joins of every kind equal
the oracle's filtered join (oracle.join_filtered with oracle.substr / oracle.str_compare)."""
import json
from pathlib import Path

import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import split

pytestmark = pytest.mark.gpu

I, L = omg.IntType(), omg.LongType()
V5 = omg.VarcharType(5)
V = omg.VarcharType(64)
F, B, Lit, Fn = omg.Field, omg.Binary, omg.Literal, omg.Func
SUBSTR = json.loads((Path(__file__).parent / "golden" / "substr_kats.json").read_text(encoding="utf-8"))


@pytest.fixture(autouse=True)
def _default_substr_rules():
    yield
    omg.set_substr_rules(1, 1)


def _value(v, m, i):
    if m[i]:
        return None
    x = v[i]
    if isinstance(x, (bytes, bytearray, np.bytes_)):
        return bytes(x)
    return float(x) if isinstance(x, np.floating) else int(x)


def run(join_type, btypes, bcols, bmasks, ptypes, pcols, pmasks, pout, bout, filt, batch_sizes=(1000,),
        build_side="UNKNOWN"):
    """Build on two builder operators, probe in ragged batches, drain the outer operator; rows as
    tuples (bytes for strings, None for NULL)."""
    kind = oracle.join_kind(join_type, build_side)
    bf = omg.HashBuilderOperatorFactory(oracle.JOIN_TYPES[join_type], btypes, [0], operator_count=2,
                                        build_side=oracle.BUILD_SIDES[build_side])
    ops = [bf.create_operator() for _ in range(2)]
    nb = len(bcols[0])
    for op, (s, e) in zip(ops, [(0, nb // 2), (nb // 2, nb)]):
        op.add_input(omg.make_batch(btypes, [c[s:e] for c in bcols], [m[s:e] for m in bmasks]))
    for op in ops:
        op.get_output()
    bo_types = [btypes[c] for c in bout]
    pf = omg.LookupJoinOperatorFactory(ptypes, pout, [0], bout, bo_types, bf, filter_expr=filt)
    pop = pf.create_operator()
    outs = []
    for s, e in split(len(pcols[0]), list(batch_sizes)):
        pop.add_input(omg.make_batch(ptypes, [c[s:e] for c in pcols], [m[s:e] for m in pmasks]))
        outs += pop.drain()
    outs += pop.drain()
    pop.delete()
    if kind in ("build_outer", "full"):
        of = omg.LookupOuterJoinOperatorFactory(ptypes, pout, bout, bo_types, bf)
        oop = of.create_operator()
        outs += oop.drain()
        oop.delete()
        of.close()
    kernel = omg.lib().omg_debug_last_probe_kernel()
    rows = []
    for b in outs:
        cols = omg.batch_to_numpy(b)
        omg.free_batch(b)
        n = len(cols[0][0]) if cols else 0
        rows += [tuple(_value(v, m, i) for v, m in cols) for i in range(n)]
    for op in ops:
        op.delete()
    pf.close()
    bf.close()
    return rows, kernel


def _key(r):
    return tuple((x is None, b"" if x is None else (x if isinstance(x, bytes) else str(x).encode())) for x in r)


def _char_filter():
    """join_test.cpp:1796-1823 (CreateJoinFilterExprWithChar): substr(#1, 1, 5) != substr(#3, 1, 5)."""
    return B(omg.EXPR_NEQ, Fn("substr", [F(1, V5), Lit(1, I), Lit(5, I)], V5),
             Fn("substr", [F(3, V5), Lit(1, I), Lit(5, I)], V5))


S1 = [b"35709", b"31904", b"35709", b"31904", b"35709", b"31904", b"35709", b"31904", b"35709", b"31904"]
S2 = [b"35709", b"35709", b"31904", b"12477", b"31904", b"38721", b"90419", b"35709", b"88371", b"35709"]
K1 = [19, 14, 7, 19, 1, 20, 10, 13, 20, 16]
K2 = [20, 16, 13, 4, 20, 4, 22, 19, 8, 7]


@pytest.mark.parametrize("case", ["CharFilter", "CharFilterWithOddDataSize", "CharFilter2",
                                  "CharFilter2WithOddDataSize"])
def test_reference_inner_join_with_char_filter(case):
    """join_test.cpp:1825-1900, 1902-1987, 1989-2064, 2066-2150: (int, varchar(5)) on both sides,
    the string column NULL at every fifth row from row 4 on the side that holds S2's strings;
    expected rows from the tests' expectations."""
    odd = case.endswith("OddDataSize")
    n = 9 if odd else 10
    if case.startswith("CharFilter2"):
        bk, bs, pk, ps = K2[:n], S2[:n], K1[:n], S1[:n]
        bnull, pnull = [i % 5 == 4 for i in range(n)], [False] * n
        want = [(19, b"31904", 19, b"35709"), (20, b"31904", 20, b"35709")] + (
            [] if odd else [(16, b"31904", 16, b"35709")])
    else:
        bk, bs, pk, ps = K1[:n], S1[:n], K2[:n], S2[:n]
        if odd:
            bk, bs = K1[:8] + [16], S1[:8] + [b"31904"]
        bnull, pnull = [False] * n, [i % 5 == 4 for i in range(n)]
        want = [(20, b"35709", 20, b"31904"), (16, b"35709", 16, b"31904"), (19, b"35709", 19, b"31904")]
    none = np.zeros(n, bool)
    rows, _ = run("INNER", [I, V5], [np.array(bk, np.int32), np.array(bs, dtype=object)], [none, np.array(bnull)],
                  [I, V5], [np.array(pk, np.int32), np.array(ps, dtype=object)], [none, np.array(pnull)], [0, 1],
                  [0, 1], _char_filter(), batch_sizes=(n,))
    assert sorted(rows, key=_key) == sorted(want, key=_key)


@pytest.mark.parametrize("rules", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("with_length", [True, False])
def test_substr_kats_on_the_probe_kernel(rules, with_length):
    """Every substr known answer of the reference (function_test.cpp) whose policy is `rules`,
    evaluated by the probe kernel: build rows hold the strings, probe rows the start, length and
    the expected result (and a wrong one); the filter substr(build.s, probe.start[, probe.len]) =
    probe.expected keeps exactly the right probe rows.  Positions as LONG columns."""
    cases = [c for k in SUBSTR.values() for c in k["cases"]
             if (int(c["negative"]), int(c["zero"])) == rules and (c["length"] is not None) == with_length]
    if not cases:
        pytest.skip("no known answer for this policy")
    omg.set_substr_rules(*rules)
    nb = len(cases)
    bkey = np.arange(nb, dtype=np.int64)
    bstr = np.array([c["string"].encode() for c in cases], dtype=object)
    pkey = np.repeat(bkey, 2)
    start = np.repeat(np.array([c["start"] for c in cases], dtype=np.int64), 2)
    length = np.repeat(np.array([c["length"] or 0 for c in cases], dtype=np.int64), 2)
    exp = np.array([x for c in cases for x in (c["expected"].encode(), c["expected"].encode() + b"~")],
                   dtype=object)
    args = [F(5, V), F(1, L)] + ([F(2, L)] if with_length else [])
    filt = B(omg.EXPR_EQ, Fn("substr", args, V), F(3, V))
    none_b, none_p = np.zeros(nb, bool), np.zeros(2 * nb, bool)
    rows, _ = run("INNER", [L, V], [bkey, bstr], [none_b, none_b], [L, L, L, V], [pkey, start, length, exp],
                  [none_p] * 4, [0, 3], [], filt, batch_sizes=(2 * nb,))
    want = [(i, c["expected"].encode()) for i, c in enumerate(cases)]
    assert sorted(rows, key=_key) == sorted(want, key=_key)


def _utf8_words(rng, n, pool):
    alphabet = ["a", "b", "c", "é", "ß", "中", "文", "😀", "z"]
    words = ["".join(rng.choice(alphabet, int(rng.integers(0, 9)))) for _ in range(pool)]
    words[0] = ""
    return np.array([words[i].encode() for i in rng.integers(0, pool, n)], dtype=object)


def _cast(x, dtype):
    """Numeric CAST (mathfunctions.cpp:24-113, RoundingRule::DOWN): integers wrap to the target
    width, DOUBLE truncates toward zero, saturating at the target's range, NaN giving 0."""
    if x is None:
        return None
    if dtype.id == omg.OMNI_DOUBLE:
        return float(x)
    bits = {omg.OMNI_LONG: 64, omg.OMNI_INT: 32, omg.OMNI_SHORT: 16}[dtype.id]
    lo, hi = -(1 << (bits - 1)), (1 << (bits - 1)) - 1
    if isinstance(x, float):
        return 0 if x != x else max(lo, min(hi, int(x)))
    return ((int(x) - lo) % (1 << bits)) + lo


def _eval(e, pcols, pmasks, bcols, bmasks, i, j, nprobe):
    """Value of filter node `e` for probe row i and build row j (None for NULL), SQL semantics."""
    if isinstance(e, omg.Field):
        probe = e.col < nprobe
        c = e.col if probe else e.col - nprobe
        cols, masks, r = (pcols, pmasks, i) if probe else (bcols, bmasks, j)
        return _value(cols[c], masks[c], r)
    if isinstance(e, omg.Literal):
        return None if e.is_null else (e.value if isinstance(e.value, (bytes, int, float)) else e.value.encode())
    if isinstance(e, omg.Func):
        a = [_eval(x, pcols, pmasks, bcols, bmasks, i, j, nprobe) for x in e.args]
        if e.name == "CAST":
            return _cast(a[0], e.dtype)
        if e.name != "substr":
            return oracle.string_function(e.name, a)
        if any(x is None for x in a):
            return None
        neg, zero = omg.get_substr_rules()
        return oracle.substr(a[0], a[1], a[2] if len(a) == 3 else None, bool(neg), bool(zero))
    if isinstance(e, omg.If):
        c = _eval(e.cond, pcols, pmasks, bcols, bmasks, i, j, nprobe)
        return _eval(e.then if c not in (None, 0) else e.else_, pcols, pmasks, bcols, bmasks, i, j, nprobe)
    if isinstance(e, omg.Switch):
        for cond, res in e.whens:
            if _eval(cond, pcols, pmasks, bcols, bmasks, i, j, nprobe) not in (None, 0):
                return _eval(res, pcols, pmasks, bcols, bmasks, i, j, nprobe)
        return _eval(e.else_, pcols, pmasks, bcols, bmasks, i, j, nprobe)
    if isinstance(e, omg.Coalesce):
        a = _eval(e.value1, pcols, pmasks, bcols, bmasks, i, j, nprobe)
        return a if a is not None else _eval(e.value2, pcols, pmasks, bcols, bmasks, i, j, nprobe)
    if isinstance(e, omg.In):
        # expression_codegen.cpp:545-659: TRUE on a match, else NULL if the value or an item is NULL
        v = _eval(e.value, pcols, pmasks, bcols, bmasks, i, j, nprobe)
        items = [_eval(x, pcols, pmasks, bcols, bmasks, i, j, nprobe) for x in e.items]
        if v is not None and any(x is not None and x == v for x in items):
            return 1
        return None if v is None or any(x is None for x in items) else 0
    if isinstance(e, omg.Between):
        # expression_codegen.cpp:661-711: NULL if any operand is NULL; doubles compare unordered as <=
        v, lo, hi = (_eval(x, pcols, pmasks, bcols, bmasks, i, j, nprobe) for x in (e.value, e.lower, e.upper))
        if v is None or lo is None or hi is None:
            return None
        if isinstance(v, bytes):
            return int(oracle.str_compare(lo, v) <= 0 and oracle.str_compare(v, hi) <= 0)
        return int(not (lo > v) and not (v > hi))
    if isinstance(e, omg.IsNull):
        return int(_eval(e.child, pcols, pmasks, bcols, bmasks, i, j, nprobe) is None)
    if isinstance(e, omg.Not):
        v = _eval(e.child, pcols, pmasks, bcols, bmasks, i, j, nprobe)
        return None if v is None else int(not v)
    a = _eval(e.left, pcols, pmasks, bcols, bmasks, i, j, nprobe)
    b = _eval(e.right, pcols, pmasks, bcols, bmasks, i, j, nprobe)
    if e.op == omg.EXPR_AND:
        if a == 0 or b == 0:
            return 0
        return None if a is None or b is None else 1
    if e.op == omg.EXPR_OR:
        if (a is not None and a != 0) or (b is not None and b != 0):
            return 1
        return None if a is None or b is None else 0
    if a is None or b is None:
        return None
    c = oracle.str_compare(a, b) if isinstance(a, bytes) else (a > b) - (a < b)
    return int({omg.EXPR_EQ: c == 0, omg.EXPR_NEQ: c != 0, omg.EXPR_LT: c < 0, omg.EXPR_LTE: c <= 0,
                omg.EXPR_GT: c > 0, omg.EXPR_GTE: c >= 0}[e.op])


D = omg.DoubleType()
NULL_V = Lit(b"", V, is_null=True)

# Probe (key, s, pos), build (key, t, payload, x): probe fields 0-2, build fields 3-6.
FILTERS = {
    "substr_lt": B(omg.EXPR_LT, Fn("substr", [F(1, V), Lit(2, I), Lit(3, I)], V),
                   Fn("substr", [F(4, V), Lit(1, I), Lit(3, I)], V)),
    "ge_or_suffix_literal": B(omg.EXPR_OR, B(omg.EXPR_GTE, F(1, V), F(4, V)),
                              B(omg.EXPR_EQ, Fn("substr", [F(4, V), Lit(-2, I)], V), Lit("a中", V))),
    "column_positions": B(omg.EXPR_EQ, Fn("substr", [F(1, V), F(2, I), Lit(2, I)], V),
                          Fn("substr", [F(4, V), Lit(1, I), Lit(2, I)], V)),
    "null_and_payload": B(omg.EXPR_AND, omg.Not(omg.IsNull(F(4, V))),
                          B(omg.EXPR_OR, B(omg.EXPR_NEQ, F(1, V), Lit(b"", V)), B(omg.EXPR_GT, F(5, L), Lit(0, L)))),
    "in_strings_and_if": B(omg.EXPR_AND,
                           omg.In(Fn("substr", [F(1, V), Lit(1, I), Lit(1, I)], V),
                                  [Lit("a", V), Lit("中", V), Lit(b"", V), F(4, V)]),
                           omg.If(B(omg.EXPR_GT, F(2, I), Lit(0, I)), B(omg.EXPR_GT, F(5, L), Lit(0, L)),
                                  B(omg.EXPR_LTE, F(5, L), Lit(0, L)))),
    "not_in_with_null_item": B(omg.EXPR_OR, omg.Not(omg.In(F(2, I), [Lit(1, I), Lit(2, I), Lit(0, I, is_null=True)])),
                               omg.Not(omg.In(F(5, L), [Lit(1, L), Lit(-1, L)]))),
    "between_case_coalesce": B(omg.EXPR_OR, omg.Between(F(6, D), Lit(-0.5, D), Lit(0.5, D)),
                               omg.Switch([(omg.IsNull(F(4, V)), B(omg.EXPR_EQ, F(2, I), Lit(0, I))),
                                           (B(omg.EXPR_GT, F(5, L), Lit(2, L)),
                                            omg.Between(F(1, V), Lit("b", V), F(4, V)))],
                                          B(omg.EXPR_EQ, omg.Coalesce(F(4, V), Lit("x", V)), Lit("x", V)))),
    "string_functions": B(omg.EXPR_OR,
                          B(omg.EXPR_AND, Fn("StartsWith", [F(1, V), Fn("substr", [F(4, V), Lit(1, I), Lit(1, I)], V)], omg.BooleanType()),
                            B(omg.EXPR_LT, Fn("length", [F(1, V)], L), Fn("instr", [F(4, V), Lit("中", V)], I))),
                          B(omg.EXPR_OR, Fn("Contains", [Fn("Greatest", [F(1, V), F(4, V)], V), Lit("ab", V)],
                                            omg.BooleanType()),
                            B(omg.EXPR_AND, Fn("EndsWith", [F(4, V), Lit("z", V)], omg.BooleanType()),
                              B(omg.EXPR_EQ, Fn("Least", [F(1, V), F(4, V)], V), F(1, V))))),
    "numeric_casts": B(omg.EXPR_OR, B(omg.EXPR_EQ, Fn("CAST", [F(6, D)], I), Fn("CAST", [F(5, L)], I)),
                       B(omg.EXPR_AND, B(omg.EXPR_GT, Fn("CAST", [F(2, I)], D), F(6, D)),
                         B(omg.EXPR_EQ, Fn("CAST", [F(5, L)], omg.ShortType()), Fn("CAST", [F(2, I)], omg.ShortType())))),
    "not_between_if": omg.Not(omg.Between(F(5, L), Lit(-2, L),
                                                  omg.If(omg.IsNull(F(6, D)), Lit(0, L), Lit(3, L)))),
}


def _string_join_data(seed, unique, nb=3000, npr=20000):
    rng = np.random.default_rng(seed)
    bkey = rng.permutation(nb).astype(np.int64) if unique else rng.integers(0, nb // 4, nb).astype(np.int64)
    bstr = _utf8_words(rng, nb, 300)
    bpay = rng.integers(-5, 5, nb).astype(np.int64)
    bx = np.where(rng.random(nb) < 0.05, np.nan, rng.normal(0, 1, nb))
    pkey = rng.integers(0, nb + nb // 5, npr).astype(np.int64)
    pstr = _utf8_words(rng, npr, 300)
    ppos = rng.integers(-6, 7, npr).astype(np.int32)
    bm = [rng.random(nb) < 0.03, rng.random(nb) < 0.1, np.zeros(nb, bool), rng.random(nb) < 0.05]
    pm = [rng.random(npr) < 0.03, rng.random(npr) < 0.1, rng.random(npr) < 0.05]
    return [bkey, bstr, bpay, bx], bm, [pkey, pstr, ppos], pm


def _expected(kind, bcols, bm, pcols, pm, pout, bout, filt):
    def passes(pi, bi):
        return np.array([_eval(filt, pcols, pm, bcols, bm, i, j, 3) in (1, True)
                         for i, j in zip(pi.tolist(), bi.tolist())], dtype=bool)

    pi, bi = oracle.join_filtered(kind, bcols[0], bm[0], pcols[0], pm[0], passes)
    want = []
    for i, j in zip(pi.tolist(), bi.tolist()):
        r = [None if i < 0 else _value(pcols[c], pm[c], i) for c in pout]
        r += [j] if kind == "existence" else [None if j < 0 else _value(bcols[c], bm[c], j) for c in bout]
        want.append(tuple(r))
    return want


@pytest.mark.parametrize("join_type,build_side", [("INNER", "UNKNOWN"), ("LEFT", "UNKNOWN"), ("FULL", "UNKNOWN"),
                                                  ("RIGHT", "RIGHT"), ("LEFT_SEMI", "UNKNOWN"),
                                                  ("LEFT_ANTI", "UNKNOWN"), ("EXISTENCE", "UNKNOWN")])
@pytest.mark.parametrize("fname", list(FILTERS))
@pytest.mark.parametrize("unique", [True, False])
def test_string_filtered_join_kinds_match_oracle(join_type, build_side, fname, unique):
    """UTF-8 strings of 0-8 code points (1- to 4-byte), empty strings and NULLs on both sides;
    string outputs on both sides; unique (ARRAY) and duplicate (HASH) builds."""
    bcols, bm, pcols, pm = _string_join_data(len(join_type) * 5 + len(fname) + unique, unique)
    kind = oracle.join_kind(join_type, build_side)
    pout = [0, 1, 2]
    bout = [] if kind in ("semi", "anti", "existence") else [1, 2]
    filt = FILTERS[fname]
    got, _ = run(join_type, [L, V, L, D], bcols, bm, [L, V, I], pcols, pm, pout, bout, filt,
                 batch_sizes=(1000, 4096, 777), build_side=build_side)
    want = _expected(kind, bcols, bm, pcols, pm, pout, bout, filt)
    assert len(want) > 0
    assert sorted(got, key=_key) == sorted(want, key=_key)


@pytest.mark.parametrize("fname", ["substr_lt", "column_positions", "between_case_coalesce"])
def test_string_filter_on_the_bitmap_probe(fname):
    """A unique ARRAY build probed in one large batch with fixed-width outputs: the bitmap kernel
    runs the string filter on each probe row's one candidate."""
    bcols, bm, pcols, pm = _string_join_data(90 + len(fname), True, nb=1 << 14, npr=300_000)
    bm[0][:] = False
    got, kernel = run("INNER", [L, V, L, D], bcols, bm, [L, V, I], pcols, pm, [0, 2], [2], FILTERS[fname],
                      batch_sizes=(300_000,))
    assert kernel == 4  # the bitmap kernel
    want = _expected("inner", bcols, bm, pcols, pm, [0, 2], [2], FILTERS[fname])
    assert len(want) > 0
    assert sorted(got, key=_key) == sorted(want, key=_key)


def test_string_function_kats_on_the_probe_kernel():
    """The reference's instr / StartsWith / EndsWith / length / Contains known answers
    (function_test.cpp:2623-2800, 3741-3797), evaluated by the probe kernel: fn(build.s[,
    probe.arg]) = probe.expected keeps the row, and a wrong expected value drops it."""
    from test_oracle_golden import STRING_FN_KATS
    got, want = set(), set()
    for name in sorted({k[0] for k in STRING_FN_KATS}):
        cases = [k for k in STRING_FN_KATS if k[0] == name]
        n = len(cases)
        ret = {"length": L, "instr": I, "char_length": I}.get(name, omg.BooleanType())
        dtype = {omg.OMNI_LONG: np.int64, omg.OMNI_INT: np.int32, omg.OMNI_BOOLEAN: np.bool_}[ret.id]
        bkey = np.arange(n, dtype=np.int64)
        bstr = np.array([k[1][0].encode() for k in cases], dtype=object)
        pkey = np.repeat(bkey, 2)
        parg = np.repeat(np.array([(k[1][1] if len(k[1]) > 1 else "").encode() for k in cases], dtype=object), 2)
        right = [k[2] for k in cases]
        wrong = [(1 - x) if ret.id == omg.OMNI_BOOLEAN else x + 7 for x in right]
        pexp = np.array([x for pair in zip(right, wrong) for x in pair], dtype=dtype)
        args = [F(4, V)] + ([F(1, V)] if len(cases[0][1]) > 1 else [])
        none_b, none_p = np.zeros(n, bool), np.zeros(2 * n, bool)
        rows, _ = run("INNER", [L, V], [bkey, bstr], [none_b, none_b], [L, V, ret], [pkey, parg, pexp],
                      [none_p] * 3, [0], [], B(omg.EXPR_EQ, Fn(name, args, ret), F(2, ret)), batch_sizes=(2 * n,))
        got |= {(name, r[0]) for r in rows}
        want |= {(name, i) for i in range(n)}
    assert got == want
