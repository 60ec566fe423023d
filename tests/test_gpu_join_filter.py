"""Join filters on the GPU: LookupJoin with a filter expression (lookup_join.cpp:175-187,
1440-1466).  A candidate pair whose keys are equal is a match only when the filter, evaluated over
the joined row (probe columns first, then build columns), is TRUE; NULL fails.  Every join kind
must equal the oracle's filtered join (oracle.join_filtered) as an exact row multiset, and the
reference's integer-filter join test must give its expected rows."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import split

pytestmark = pytest.mark.gpu

L, I, D = omg.LongType(), omg.IntType(), omg.DoubleType()
F, B = omg.Field, omg.Binary


def _rows(batches):
    rows = []
    for b in batches:
        cols = omg.batch_to_numpy(b)
        omg.free_batch(b)
        n = len(cols[0][0]) if cols else 0
        for i in range(n):
            rows.append(tuple(None if m[i] else (float(v[i]) if isinstance(v[i], np.floating) else int(v[i]))
                              for v, m in cols))
    return rows


def run(join_type, build_side, btypes, bcols, bmasks, ptypes, pcols, pmasks, pout, bout, filt,
        batch_sizes=(1000,)):
    """Build on two builder operators, probe in ragged batches, drain the outer-join operator."""
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
    rows = _rows(outs)
    if kind in ("build_outer", "full"):
        of = omg.LookupOuterJoinOperatorFactory(ptypes, pout, bout, bo_types, bf)
        oop = of.create_operator()
        rows += _rows(oop.drain())
        oop.delete()
        of.close()
    for op in ops:
        op.delete()
    pf.close()
    bf.close()
    return rows


def _key(r):
    return tuple((x is None, 0 if x is None else x) for x in r)


@pytest.mark.parametrize("odd", [False, True])
def test_reference_inner_join_with_int_filter(odd):
    """join_test.cpp:1545-1625 (TestInnerEqualityJoinWithIntFilter) and :1627-1705 (its odd-size
    twin with an 11th row on both sides): build (int, int), probe (int, int) with the probe's second
    column NULL at every fifth row from row 4, filter #1 != #3; expected rows
    (20, 35709, 20, 31904), (16, 35709, 16, 31904), (19, 35709, 19, 31904)."""
    b0 = [19, 14, 7, 19, 1, 20, 10, 13, 20, 16] + ([15] if odd else [])
    b1 = [35709, 31904, 35709, 31904, 35709, 31904, 35709, 31904, 35709, 31904] + ([31904] if odd else [])
    p0 = [20, 16, 13, 4, 20, 4, 22, 19, 8, 7] + ([11] if odd else [])
    p1 = [35709, 35709, 31904, 12477, 31904, 38721, 90419, 35709, 88371, 35709] + ([35709] if odd else [])
    n = len(p0)
    b0, b1, p0, p1 = (np.array(x, dtype=np.int32) for x in (b0, b1, p0, p1))
    pm = np.array([i % 5 == 4 for i in range(n)])
    none = np.zeros(n, bool)
    filt = B(omg.EXPR_NEQ, F(1, I), F(3, I))
    rows = run("INNER", "UNKNOWN", [I, I], [b0, b1], [none, none], [I, I], [p0, p1], [none, pm], [0, 1], [0, 1],
               filt, batch_sizes=(n,))
    assert sorted(rows) == sorted([(20, 35709, 20, 31904), (16, 35709, 16, 31904), (19, 35709, 19, 31904)])


def _eval(e, pi, bi, pcols, pmasks, bcols, bmasks):
    """(values, null mask, is_double) of expression `e` over candidate pairs, SQL three-valued."""
    n_probe = len(pcols)
    if isinstance(e, omg.Field):
        probe = e.col < n_probe
        c = e.col if probe else e.col - n_probe
        rows = pi if probe else bi
        col, m = (pcols[c], pmasks[c]) if probe else (bcols[c], bmasks[c])
        return col[rows], m[rows].copy(), col.dtype.kind == "f"
    if isinstance(e, omg.Literal):
        dbl = e.dtype.id == omg.OMNI_DOUBLE
        v = np.full(len(pi), float(e.value) if dbl else int(e.value), dtype=np.float64 if dbl else np.int64)
        return v, np.full(len(pi), bool(e.is_null)), dbl
    if isinstance(e, omg.Not):
        v, m, _ = _eval(e.child, pi, bi, pcols, pmasks, bcols, bmasks)
        return (v == 0).astype(np.int64), m, False
    if isinstance(e, omg.IsNull):
        _, m, _ = _eval(e.child, pi, bi, pcols, pmasks, bcols, bmasks)
        return m.astype(np.int64), np.zeros(len(pi), bool), False
    a, am, ad = _eval(e.left, pi, bi, pcols, pmasks, bcols, bmasks)
    b, bm, bd = _eval(e.right, pi, bi, pcols, pmasks, bcols, bmasks)
    if e.op >= omg.EXPR_ADD:
        return _arith(e, a, am, ad, b, bm, bd)
    if e.op == omg.EXPR_AND:
        af, bf_ = ~am & (a == 0), ~bm & (b == 0)
        null = ~(af | bf_) & (am | bm)
        return (~af & ~bf_ & ~null).astype(np.int64), null, False
    if e.op == omg.EXPR_OR:
        at, bt = ~am & (a != 0), ~bm & (b != 0)
        null = ~(at | bt) & (am | bm)
        return (at | bt).astype(np.int64), null, False
    if ad or bd:
        a, b = a.astype(np.float64), b.astype(np.float64)
    cmp = {omg.EXPR_EQ: a == b, omg.EXPR_NEQ: a != b, omg.EXPR_LT: a < b, omg.EXPR_LTE: a <= b,
           omg.EXPR_GT: a > b, omg.EXPR_GTE: a >= b}[e.op]
    return cmp.astype(np.int64), am | bm, False


def _arith(e, a, am, ad, b, bm, bd):
    """The reference's math functions (codegen/functions/mathfunctions.cpp) in Python numbers:
    integers wrap at the node's width, DIV / MOD by zero are NULL, TRY_* overflow is NULL (TRY_DIV
    is DIV), doubles are IEEE with fmod; C division truncates toward zero."""
    null = am | bm
    if e.dtype.id == omg.OMNI_DOUBLE:
        x, y = a.astype(np.float64), b.astype(np.float64)
        with np.errstate(all="ignore"):
            if e.op in (omg.EXPR_ADD, omg.EXPR_TRY_ADD):
                r = x + y
            elif e.op in (omg.EXPR_SUB, omg.EXPR_TRY_SUB):
                r = x - y
            elif e.op in (omg.EXPR_MUL, omg.EXPR_TRY_MUL):
                r = x * y
            else:
                zero = y == 0
                null = null | zero
                r = np.where(zero, 0.0, np.fmod(x, np.where(zero, 1.0, y)) if e.op == omg.EXPR_MOD
                             else x / np.where(zero, 1.0, y))
        return r, null, True
    bits = 8 * (4 if e.dtype.id == omg.OMNI_INT else 8)
    lo, hi = -(1 << (bits - 1)), (1 << (bits - 1)) - 1
    out = np.zeros(len(a), dtype=np.int64)
    for i, (x, y) in enumerate(zip(a.tolist(), b.tolist())):
        if null[i]:
            continue
        x, y = int(x), int(y)
        if e.op in (omg.EXPR_DIV, omg.EXPR_TRY_DIV, omg.EXPR_MOD):
            if y == 0:
                null[i] = True
                continue
            q = abs(x) // abs(y) * (1 if (x >= 0) == (y > 0) else -1)
            r = q if e.op != omg.EXPR_MOD else x - q * y
        else:
            r = {omg.EXPR_ADD: x + y, omg.EXPR_TRY_ADD: x + y, omg.EXPR_SUB: x - y, omg.EXPR_TRY_SUB: x - y,
                 omg.EXPR_MUL: x * y, omg.EXPR_TRY_MUL: x * y}[e.op]
            if not lo <= r <= hi and e.op in (omg.EXPR_TRY_ADD, omg.EXPR_TRY_SUB, omg.EXPR_TRY_MUL):
                null[i] = True
                continue
        out[i] = ((r - lo) % (1 << bits)) + lo  # wrap at the width
    return out, null, False


def _passes(e, pcols, pmasks, bcols, bmasks):
    def f(pi, bi):
        v, m, _ = _eval(e, pi, bi, pcols, pmasks, bcols, bmasks)
        return (v != 0) & ~m
    return f


FILTERS = {
    "int_lt": B(omg.EXPR_LT, F(1, L), F(4, L)),
    "double_or_null": B(omg.EXPR_OR, B(omg.EXPR_GTE, F(2, D), F(5, D)), omg.IsNull(F(4, L))),
    "not_eq_and_literal": B(omg.EXPR_AND, omg.Not(B(omg.EXPR_EQ, F(1, L), F(4, L))),
                            B(omg.EXPR_GT, F(2, D), omg.Literal(0.25, D))),
    "build_only_and_null_literal": B(omg.EXPR_OR, B(omg.EXPR_GTE, F(4, L), omg.Literal(0, L)),
                                     B(omg.EXPR_EQ, F(1, L), omg.Literal(0, L, is_null=True))),
    "arith_add_div_mod": B(omg.EXPR_AND, B(omg.EXPR_LT, B(omg.EXPR_ADD, F(1, L), F(4, L), L), omg.Literal(3, L)),
                           B(omg.EXPR_NEQ, B(omg.EXPR_MOD, F(1, L), F(4, L), L),
                             B(omg.EXPR_DIV, F(4, L), omg.Literal(3, L), L))),
    "arith_double_and_try": B(omg.EXPR_OR, B(omg.EXPR_GT, B(omg.EXPR_SUB, B(omg.EXPR_MUL, F(2, D),
                                                                           omg.Literal(2.0, D), D),
                                                         F(5, D), D), omg.Literal(0.5, D)),
                              omg.IsNull(B(omg.EXPR_TRY_MUL, F(1, L), omg.Literal(1 << 62, L), L))),
}


@pytest.mark.parametrize("join_type,build_side", [("INNER", "UNKNOWN"), ("LEFT", "UNKNOWN"), ("FULL", "UNKNOWN"),
                                                  ("RIGHT", "RIGHT"), ("LEFT_SEMI", "UNKNOWN"),
                                                  ("LEFT_ANTI", "UNKNOWN"), ("EXISTENCE", "UNKNOWN")])
@pytest.mark.parametrize("fname", list(FILTERS))
@pytest.mark.parametrize("unique", [True, False])
def test_filtered_join_kinds_match_oracle(join_type, build_side, fname, unique):
    rng = np.random.default_rng(len(join_type) * 13 + len(fname) + unique)
    nb, npr = 3000, 20000
    bkey = rng.permutation(nb).astype(np.int64) if unique else rng.integers(0, nb // 4, nb).astype(np.int64)
    bv = rng.integers(-20, 20, nb).astype(np.int64)
    bd = rng.random(nb)
    bm = [rng.random(nb) < 0.03, rng.random(nb) < 0.1, rng.random(nb) < 0.1]
    pkey = rng.integers(0, nb + nb // 5, npr).astype(np.int64)
    pv = rng.integers(-20, 20, npr).astype(np.int64)
    pd = rng.random(npr)
    pm = [rng.random(npr) < 0.03, rng.random(npr) < 0.1, rng.random(npr) < 0.1]
    bcols, pcols = [bkey, bv, bd], [pkey, pv, pd]
    kind = oracle.join_kind(join_type, build_side)
    pout = [0, 1, 2]
    bout = [] if kind in ("semi", "anti", "existence") else [1, 2]
    filt = FILTERS[fname]
    got = run(join_type, build_side, [L, L, D], bcols, bm, [L, L, D], pcols, pm, pout, bout, filt,
              batch_sizes=(1000, 4096, 777))
    pi, bi = oracle.join_filtered(kind, bkey, bm[0], pkey, pm[0], _passes(filt, pcols, pm, bcols, bm))

    def val(cols, masks, c, r):
        if r < 0 or masks[c][r]:
            return None
        v = cols[c][r]
        return float(v) if isinstance(v, np.floating) else int(v)

    want = []
    for i, j in zip(pi.tolist(), bi.tolist()):
        r = [val(pcols, pm, c, i) for c in pout]
        r += [j] if kind == "existence" else [val(bcols, bm, c, j) for c in bout]
        want.append(tuple(r))
    assert len(want) > 0
    assert sorted(got, key=_key) == sorted(want, key=_key)


def test_int_arithmetic_wraps_at_32_bits():
    """INT arithmetic wraps at 32 bits (AddInt32, MultiplyInt32) while TRY_ADD gives NULL on
    overflow: pairs with p + b beyond 2^31 - 1 wrap negative, so `p + b < 0` holds for them, and
    `TRY_ADD(p, b) IS NULL` marks the same pairs."""
    n = 200
    key = np.arange(n, dtype=np.int64)
    pv = np.array([2**31 - 1 - (i % 7) for i in range(n)], dtype=np.int32)
    bv = np.array([i % 11 for i in range(n)], dtype=np.int32)
    none = np.zeros(n, bool)
    for filt in (B(omg.EXPR_LT, B(omg.EXPR_ADD, F(1, I), F(3, I), I), omg.Literal(0, I)),
                 omg.IsNull(B(omg.EXPR_TRY_ADD, F(1, I), F(3, I), I))):
        rows = run("INNER", "UNKNOWN", [L, I], [key, bv], [none, none], [L, I], [key, pv], [none, none], [0, 1],
                   [1], filt, batch_sizes=(n,))
        want = sorted((int(k), int(p), int(b)) for k, p, b in zip(key, pv, bv) if int(p) + int(b) > 2**31 - 1)
        assert len(want) > 0 and sorted(rows) == want


@pytest.mark.parametrize("join_type", ["INNER", "LEFT", "LEFT_SEMI", "LEFT_ANTI", "EXISTENCE"])
@pytest.mark.parametrize("fname", list(FILTERS))
def test_filtered_bitmap_probe_matches_oracle(join_type, fname):
    """A unique ARRAY build probed in one large batch: the bitmap kernel evaluates the filter on
    each probe row's one candidate (its slot's build row) and must equal the oracle's filtered
    join; build output columns are NULL-free so that they come from the packed slot payload."""
    rng = np.random.default_rng(len(join_type) * 7 + len(fname))
    nb, npr = 1 << 15, 300_000
    bkey = rng.permutation(nb).astype(np.int64)
    bv = rng.integers(-20, 20, nb).astype(np.int64)
    bd = rng.random(nb)
    bw = rng.integers(-2**31, 2**31, nb, dtype=np.int64).astype(np.int32)
    bm = [np.zeros(nb, bool), rng.random(nb) < 0.1, rng.random(nb) < 0.1, np.zeros(nb, bool)]
    pkey = rng.integers(0, nb + nb // 5, npr).astype(np.int64)
    pv = rng.integers(-20, 20, npr).astype(np.int64)
    pd = rng.random(npr)
    pm = [rng.random(npr) < 0.03, rng.random(npr) < 0.1, rng.random(npr) < 0.1]
    bcols, pcols = [bkey, bv, bd, bw], [pkey, pv, pd]
    kind = oracle.join_kind(join_type, "UNKNOWN")
    pout = [0, 1, 2]
    bout = [] if kind in ("semi", "anti", "existence") else [3]
    filt = FILTERS[fname]
    got = run(join_type, "UNKNOWN", [L, L, D, I], bcols, bm, [L, L, D], pcols, pm, pout, bout, filt,
              batch_sizes=(npr,))
    assert omg.lib().omg_debug_last_probe_kernel() == 4  # the bitmap kernel
    pi, bi = oracle.join_filtered(kind, bkey, bm[0], pkey, pm[0], _passes(filt, pcols, pm, bcols, bm))

    def val(cols, masks, c, r):
        if r < 0 or masks[c][r]:
            return None
        v = cols[c][r]
        return float(v) if isinstance(v, np.floating) else int(v)

    want = []
    for i, j in zip(pi.tolist(), bi.tolist()):
        r = [val(pcols, pm, c, i) for c in pout]
        r += [j] if kind == "existence" else [val(bcols, bm, c, j) for c in bout]
        want.append(tuple(r))
    assert len(want) > 0
    assert sorted(got, key=_key) == sorted(want, key=_key)


@pytest.mark.parametrize("fop,lit", [(omg.EXPR_GTE, 0), (omg.EXPR_LT, -5), (omg.EXPR_NEQ, 7)])
def test_filter_on_payload_fields_headline_layout(fop, lit):
    """The headline shape (8-byte probe key out, two int32 build payload fields out) with one
    comparison on a payload field: the bitmap kernel's compile-time layout evaluates it from the
    slot payload; rows against a direct restatement."""
    rng = np.random.default_rng(60 + fop)
    nb, npr = 1 << 16, 400_000
    bkey = rng.permutation(nb).astype(np.int64)
    p1 = rng.integers(-20, 20, nb).astype(np.int32)
    p2 = rng.integers(-2**31, 2**31, nb, dtype=np.int64).astype(np.int32)
    pkey = rng.integers(0, nb + nb // 4, npr).astype(np.int64)
    pm = rng.random(npr) < 0.01
    none_b = np.zeros(nb, bool)
    filt = B(fop, F(2, I), omg.Literal(lit, I))
    got = run("INNER", "UNKNOWN", [L, I, I], [bkey, p1, p2], [none_b, none_b, none_b], [L], [pkey], [pm], [0], [1, 2],
              filt, batch_sizes=(npr,))
    assert omg.lib().omg_debug_last_probe_kernel() == 4
    pos = np.full(nb + nb // 4, -1, np.int64)
    pos[bkey] = np.arange(nb)
    bi = pos[pkey]
    ok = (bi >= 0) & ~pm
    cmp = {omg.EXPR_GTE: np.greater_equal, omg.EXPR_LT: np.less, omg.EXPR_NEQ: np.not_equal}[fop]
    ok &= cmp(p1[np.where(ok, bi, 0)].astype(np.int64), lit)
    want = sorted(zip(pkey[ok].tolist(), p1[bi[ok]].tolist(), p2[bi[ok]].tolist()))
    assert len(want) > 0 and sorted(got) == want


@pytest.mark.parametrize("fop", [omg.EXPR_LT, omg.EXPR_GTE, omg.EXPR_EQ])
@pytest.mark.parametrize("probe_first", [True, False])
def test_filter_probe_column_against_payload_field(fop, probe_first):
    """The headline shape with one comparison between a probe column (INT, with NULLs) and a build
    payload field, in either order: the bitmap kernel decodes the comparison once and reads the
    field from the slot payload; rows against a direct restatement (a NULL probe value fails)."""
    rng = np.random.default_rng(70 + fop + 3 * probe_first)
    nb, npr = 1 << 16, 400_000
    bkey = rng.permutation(nb).astype(np.int64)
    p1 = rng.integers(-20, 20, nb).astype(np.int32)
    p2 = rng.integers(-2**31, 2**31, nb, dtype=np.int64).astype(np.int32)
    pkey = rng.integers(0, nb + nb // 4, npr).astype(np.int64)
    pv = rng.integers(-20, 20, npr).astype(np.int32)
    pm, vm = rng.random(npr) < 0.01, rng.random(npr) < 0.05
    none_b = np.zeros(nb, bool)
    a, b = (F(1, I), F(3, I)) if probe_first else (F(3, I), F(1, I))
    got = run("INNER", "UNKNOWN", [L, I, I], [bkey, p1, p2], [none_b, none_b, none_b], [L, I], [pkey, pv], [pm, vm],
              [0], [1, 2], B(fop, a, b), batch_sizes=(npr,))
    assert omg.lib().omg_debug_last_probe_kernel() == 4
    pos = np.full(nb + nb // 4, -1, np.int64)
    pos[bkey] = np.arange(nb)
    bi = pos[pkey]
    ok = (bi >= 0) & ~pm & ~vm
    x = pv.astype(np.int64)
    y = p1[np.where(ok, bi, 0)].astype(np.int64)
    if not probe_first:
        x, y = y, x
    cmp = {omg.EXPR_GTE: np.greater_equal, omg.EXPR_LT: np.less, omg.EXPR_EQ: np.equal}[fop]
    ok &= cmp(x, y)
    want = sorted(zip(pkey[ok].tolist(), p1[bi[ok]].tolist(), p2[bi[ok]].tolist()))
    assert len(want) > 0 and sorted(got) == want
