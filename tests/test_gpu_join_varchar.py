"""VARCHAR in the join: string keys (alone and with an integer key column), string payloads on
both sides, every join kind, against the oracle on random inputs and against the reference's
join tests that use VARCHAR payloads (join_test.cpp:3831-3889, 4014-4081) with their original
strings.  Rows compared as exact multisets (strings as bytes, NULL as None)."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import split, tuple_ids

pytestmark = pytest.mark.gpu

L, I, V = omg.LongType(), omg.IntType(), omg.VarcharType(64)


def _batch(types, cols, masks):
    return omg.make_batch(types, cols, masks)


def _rows_of(batches):
    rows = []
    for b in batches:
        cols = omg.batch_to_numpy(b)
        omg.free_batch(b)
        for i in range(len(cols[0][0]) if cols else 0):
            rows.append(tuple(None if m[i] else (bytes(v[i]) if isinstance(v[i], (bytes, bytearray))
                                                 else int(v[i])) for v, m in cols))
    return rows


def _key(r):
    return tuple((x is None, b"" if x is None else (x if isinstance(x, bytes) else str(x).encode())) for x in r)


def run_join(join_type, build_side, btypes, bcols, bmasks, bhash, ptypes, pcols, pmasks, phash, pout, bout,
             batch_sizes=(1000,)):
    kind = oracle.join_kind(join_type, build_side)
    bf = omg.HashBuilderOperatorFactory(oracle.JOIN_TYPES[join_type], btypes, bhash, operator_count=2,
                                        build_side=oracle.BUILD_SIDES[build_side])
    ops = [bf.create_operator() for _ in range(2)]
    nb = len(bcols[0])
    half = nb // 2
    for op, (s, e) in zip(ops, [(0, half), (half, nb)]):
        op.add_input(_batch(btypes, [c[s:e] for c in bcols], [m[s:e] for m in bmasks]))
    for op in ops:
        op.get_output()
    bo_types = [btypes[c] for c in bout]
    pf = omg.LookupJoinOperatorFactory(ptypes, pout, phash, bout, bo_types, bf)
    pop = pf.create_operator()
    outs = []
    for s, e in split(len(pcols[0]), list(batch_sizes)):
        pop.add_input(_batch(ptypes, [c[s:e] for c in pcols], [m[s:e] for m in pmasks]))
        outs += pop.drain()
    outs += pop.drain()
    pop.delete()
    rows = _rows_of(outs)
    outer = []
    if kind in ("build_outer", "full"):
        of = omg.LookupOuterJoinOperatorFactory(ptypes, pout, bout, bo_types, bf)
        oop = of.create_operator()
        outer = _rows_of(oop.drain())
        oop.delete()
        of.close()
    for op in ops:
        op.delete()
    pf.close()
    bf.close()
    return rows, outer


def _val(col, mask, i):
    if i < 0 or mask[i]:
        return None
    v = col[i]
    return bytes(v) if isinstance(v, (bytes, bytearray)) else int(v)


def expected(kind, bcols, bmasks, bhash, pcols, pmasks, phash, pout, bout):
    def ids(cols, masks, hashes):
        return [cols[c] for c in hashes], [masks[c] for c in hashes]
    bk, bm = ids(bcols, bmasks, bhash)
    pk, pm = ids(pcols, pmasks, phash)
    # strings become dense ids shared by both sides, then tuples become ids
    bk2, pk2 = [], []
    for x, y in zip(bk, pk):
        if x.dtype == object:
            d = {}
            bk2.append(np.array([d.setdefault(bytes(v), len(d)) for v in x], dtype=np.int64))
            pk2.append(np.array([d.setdefault(bytes(v), len(d)) for v in y], dtype=np.int64))
        else:
            bk2.append(x)
            pk2.append(y)
    bid, bn, pid, pn = tuple_ids(bk2, bm, pk2, pm)
    pi, bi = oracle.join(kind, bid, bn, pid, pn)
    rows, outer = [], []
    for i, j in zip(pi.tolist(), bi.tolist()):
        r = [_val(pcols[c], pmasks[c], i) for c in pout]
        r += [j] if kind == "existence" else [_val(bcols[c], bmasks[c], j) for c in bout]
        (outer if i < 0 else rows).append(tuple(r))
    return rows, outer


def _strings(rng, n, pool):
    lens = rng.integers(0, 40, pool)
    words = [bytes(rng.integers(97, 123, l, dtype=np.uint8)) for l in lens]
    words[0] = b""  # the empty string is a value, distinct from NULL
    idx = rng.integers(0, pool, n)
    return np.array([words[i] for i in idx], dtype=object), idx


@pytest.mark.parametrize("join_type,build_side", [("INNER", "UNKNOWN"), ("LEFT", "UNKNOWN"), ("FULL", "UNKNOWN"),
                                                  ("RIGHT", "RIGHT"), ("LEFT_SEMI", "UNKNOWN"),
                                                  ("LEFT_ANTI", "UNKNOWN"), ("EXISTENCE", "UNKNOWN")])
@pytest.mark.parametrize("keys", ["varchar", "varchar_long"])
def test_varchar_keys_and_payloads_match_oracle(join_type, build_side, keys):
    rng = np.random.default_rng(len(join_type) * 7 + len(keys))
    nb, npr, pool = 6000, 20000, 3000
    bstr, bidx = _strings(rng, nb, pool)
    pstr, pidx = _strings(rng, npr, pool)
    bnum = (bidx % 5).astype(np.int64)
    pnum = (pidx % 5).astype(np.int64)
    bpay = np.array([b"p" + bytes(str(i), "ascii") for i in range(nb)], dtype=object)
    bpay_i = rng.integers(-1000, 1000, nb).astype(np.int32)
    ppay = np.array([b"q" * (i % 7) for i in range(npr)], dtype=object)
    bm = [rng.random(nb) < 0.03, np.zeros(nb, bool), rng.random(nb) < 0.1, rng.random(nb) < 0.1]
    pm = [rng.random(npr) < 0.03, np.zeros(npr, bool), rng.random(npr) < 0.1]
    bcols = [bstr, bnum, bpay, bpay_i]
    pcols = [pstr, pnum, ppay]
    btypes, ptypes = [V, L, V, I], [V, L, V]
    hashes = [0] if keys == "varchar" else [0, 1]
    kind = oracle.join_kind(join_type, build_side)
    pout = [0, 2, 1]
    bout = [] if kind in ("semi", "anti", "existence") else [2, 3, 0]
    got, got_outer = run_join(join_type, build_side, btypes, bcols, bm, hashes, ptypes, pcols, pm, hashes, pout, bout,
                              batch_sizes=(1000, 4096, 777))
    want, want_outer = expected(kind, bcols, bm, hashes, pcols, pm, hashes, pout, bout)
    assert len(got) == len(want) > 0
    assert sorted(got, key=_key) == sorted(want, key=_key)
    assert sorted(got_outer, key=_key) == sorted(want_outer, key=_key)


def test_reference_left_semi_join_with_varchar_payload():
    """join_test.cpp:3831-3889 as written: VARCHAR(3) build payload, VARCHAR(2) probe payload."""
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_LEFT_SEMI, [L, omg.VarcharType(3)], [0])
    bop = bf.create_operator()
    bk = np.array([1, 0, 3, 0, 1, 0, 2, 2], dtype=np.int64)
    bop.add_input(_batch([L, omg.VarcharType(3)], [bk, ["aaa", "11", "ccc", "33", "aaa", "11", "ccc", "33"]],
                         [np.array([0, 1, 0, 0, 0, 0, 0, 0], bool), None]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L, omg.VarcharType(2)], [0, 1], [0], [], [], bf)
    pop = pf.create_operator()
    pk = np.array([0, 2, 0, 1, 0, 2, 0, 4], dtype=np.int64)
    pop.add_input(_batch([L, omg.VarcharType(2)], [pk, ["11", "22", "33", "44", "11", "22", "33", "44"]],
                         [np.array([0, 0, 1, 0, 0, 0, 0, 0], bool), None]))
    rows = _rows_of(pop.drain())
    want = [(0, b"11"), (2, b"22"), (1, b"44"), (0, b"11"), (2, b"22"), (0, b"33")]
    assert sorted(rows, key=_key) == sorted(want, key=_key)
    pop.delete()
    bop.delete()
    pf.close()
    bf.close()


def test_reference_right_join_with_varchar_payloads():
    """join_test.cpp:4014-4081 as written: a RIGHT join without a build side keeps unmatched
    probe rows; VARCHAR payloads on both sides."""
    V3, V2 = omg.VarcharType(3), omg.VarcharType(2)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_RIGHT, [L, V3], [0])
    bop = bf.create_operator()
    bop.add_input(_batch([L, V3], [np.array([1, 0, 3, 0, 1, 0, 2, 2], dtype=np.int64),
                                   ["aaa", "11", "ccc", "33", "aa", "11", "ccc", "33"]], None))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L, V2], [0, 1], [0], [0, 1], [L, V3], bf)
    pop = pf.create_operator()
    pop.add_input(_batch([L, V2], [np.array([0, 2, 0, 1], dtype=np.int64), ["11", "22", "33", "44"]],
                         [np.array([0, 0, 1, 0], bool), None]))
    rows = _rows_of(pop.drain())
    want = [(0, b"11", 0, b"11"), (0, b"11", 0, b"33"), (0, b"11", 0, b"11"), (2, b"22", 2, b"ccc"),
            (2, b"22", 2, b"33"), (1, b"44", 1, b"aaa"), (1, b"44", 1, b"aa"), (None, b"33", None, None)]
    assert sorted(rows, key=_key) == sorted(want, key=_key)
    pop.delete()
    bop.delete()
    pf.close()
    bf.close()
