"""Join types other than inner on the GPU: left/right/full outer joins (unmatched probe rows or,
through the LookupOuterJoin operator, unmatched build rows), left semi, left anti and existence
joins.  Checked against the reference's own join tests (tests/golden/join_type_kats.json) and
against the oracle on random inputs, row multisets compared exactly."""
import json
from pathlib import Path

import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import kat_columns, kat_hash_cols, row_key, rows_matrix, split, tuple_ids

pytestmark = pytest.mark.gpu

JOIN_TYPED = json.loads((Path(__file__).parent / "golden" / "join_type_kats.json").read_text())
L, I, S = omg.LongType(), omg.IntType(), omg.ShortType()


def _columns(batches):
    cols = None
    for b in batches:
        c = omg.batch_to_numpy(b)
        omg.free_batch(b)
        cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                       for a, x in zip(cols, c)]
    return cols


def run_typed_join(join_type, build_side, build_types, build_cols, build_masks, bhash, probe_types, probe_cols,
                   probe_masks, phash, probe_out, build_out, batch_sizes=(4096,), build_batches=1,
                   pipeline=False, outer_side=omg.OMNI_BUILD_UNKNOWN):
    """(probe operator output columns, outer-join operator output columns or None, number of
    outer output batches).  Probe output of a build-left join is rotated back to probe-first."""
    kind = oracle.join_kind(join_type, build_side)
    jt, bs = oracle.JOIN_TYPES[join_type], oracle.BUILD_SIDES[build_side]
    bhash = bhash if isinstance(bhash, list) else [bhash]
    phash = phash if isinstance(phash, list) else [phash]
    bf = omg.HashBuilderOperatorFactory(jt, build_types, bhash, operator_count=build_batches, build_side=bs)
    builders = [bf.create_operator() for _ in range(build_batches)]
    nb = len(build_cols[0])
    step = -(-nb // build_batches) if nb else 1
    for i, bop in enumerate(builders):
        s, e = min(nb, i * step), min(nb, (i + 1) * step)
        if e > s:
            bop.add_input(omg.make_batch(build_types, [c[s:e] for c in build_cols], [m[s:e] for m in build_masks]))
    for bop in builders:
        bop.get_output()
        assert bop.get_status() == omg.OMNI_STATUS_FINISHED
    bo_types = [build_types[c] for c in build_out]
    pf = omg.LookupJoinOperatorFactory(probe_types, probe_out, phash, build_out, bo_types, bf)
    pop = pf.create_operator()
    assert not pop.is_blocked()
    outs = []
    if pipeline:
        pop.set_no_more_input(False)
    for s, e in split(len(probe_cols[0]), list(batch_sizes)):
        pop.add_input(omg.make_batch(probe_types, [c[s:e] for c in probe_cols], [m[s:e] for m in probe_masks]))
        if not pipeline:
            outs += pop.drain()
    if pipeline:
        outs += pop.drain()
        pop.no_more_input()
    outs += pop.drain()
    assert pop.get_status() == omg.OMNI_STATUS_FINISHED
    pop.delete()
    cols = _columns(outs)
    if cols is not None and build_side == "LEFT":
        n = len(probe_out)
        cols = cols[len(cols) - n:] + cols[:len(cols) - n]
    outer, n_outer = None, 0
    if kind in ("build_outer", "full"):
        of = omg.LookupOuterJoinOperatorFactory(probe_types, probe_out, build_out, bo_types, bf, build_side=outer_side)
        oop = of.create_operator()
        obatches = oop.drain()
        assert oop.get_status() == omg.OMNI_STATUS_FINISHED
        n_outer = len(obatches)
        outer = _columns(obatches)
        if outer is not None and outer_side == omg.OMNI_BUILD_LEFT:
            n = len(probe_out)
            outer = outer[len(outer) - n:] + outer[:len(outer) - n]
        oop.delete()
        of.close()
    for bop in builders:
        bop.delete()
    pf.close()
    bf.close()
    return cols, outer, n_outer


def _rows(cols):
    if cols is None:
        return []
    out = []
    for i in range(len(cols[0][0])):
        out.append([None if m[i] else int(v[i]) for v, m in cols])
    return out


@pytest.mark.parametrize("name", sorted(JOIN_TYPED))
def test_join_type_kats_on_gpu(name):
    """The reference's own outer/semi/anti/existence join tests, row multisets compared."""
    k = JOIN_TYPED[name]
    (b, bm), (p, pm) = kat_columns(k)
    t = k.get("types", "LONG")
    types = [{"SHORT": S, "INT": I, "LONG": L}[x] for x in (t if isinstance(t, list) else [t] * len(b))]
    cols, outer, _ = run_typed_join(k["join_type"], k["build_side"], types, b, bm, kat_hash_cols(k, "build"),
                                    types, p, pm, kat_hash_cols(k, "probe"), k["probe_output_cols"],
                                    k["build_output_cols"])
    assert sorted(map(row_key, _rows(cols))) == sorted(map(row_key, k["expected_rows"]))
    if k["outer_rows"] is not None:
        assert sorted(map(row_key, _rows(outer))) == sorted(map(row_key, k["outer_rows"]))


def test_existence_column_is_boolean():
    k = JOIN_TYPED["existence_join"]
    (b, bm), (p, pm) = kat_columns(k)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_EXISTENCE, [L, L], [1])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, L], b))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L, L], [0], [1], [], [], bf)
    pop = pf.create_operator()
    pop.add_input(omg.make_batch([L, L], p))
    (out,) = pop.drain()
    lib = omg.lib()
    assert lib.omg_vec_type(lib.omg_batch_get(out, 1)) == omg.OMNI_BOOLEAN
    (keys, _), (flags, fm) = omg.batch_to_numpy(out)
    assert keys.tolist() == [1, 2, 3, 4, 3, 6] and flags.astype(int).tolist() == [1, 0, 1, 0, 0, 0] and not fm.any()
    omg.free_batch(out)
    pop.delete()
    bop.delete()
    pf.close()
    bf.close()


def _random_join_input(n_build, n_probe, dense, dup, seed):
    rng = np.random.default_rng(seed)
    if dense:
        domain = np.arange(1000, 1000 + n_build * 2, dtype=np.int64)
    else:
        domain = rng.choice(np.arange(-2**50, 2**50, 2**20 + 7, dtype=np.int64), n_build * 2, replace=False)
    if dup:
        bkey = domain[rng.integers(0, n_build // 3, n_build)]
    else:
        bkey = rng.permutation(domain[:n_build])
    bnull = rng.random(n_build) < 0.02
    b1 = rng.integers(-2**31, 2**31, n_build, dtype=np.int64).astype(np.int32)
    b1n = rng.random(n_build) < 0.05
    b2 = rng.integers(-2**62, 2**62, n_build, dtype=np.int64)
    pkey = domain[rng.integers(0, len(domain), n_probe)]
    pnull = rng.random(n_probe) < 0.02
    p1 = rng.integers(-2**31, 2**31, n_probe, dtype=np.int64).astype(np.int32)
    p1n = rng.random(n_probe) < 0.05
    return ([bkey, b1, b2], [bnull, b1n, np.zeros(n_build, bool)],
            [pkey, p1], [pnull, p1n])


def _expected_cols(kind, bcols, bmasks, pcols, pmasks, probe_out, build_out):
    pi, bi = oracle.join(kind, bcols[0], bmasks[0], pcols[0], pmasks[0])
    inner = pi >= 0 if kind in ("build_outer", "full") else np.ones(len(pi), bool)
    cols = []
    for c in probe_out:
        ok = pi >= 0
        idx = np.where(ok, pi, 0)
        cols.append((pcols[c][idx], ~ok | pmasks[c][idx]))
    if kind == "existence":
        cols.append((bi, np.zeros(len(bi), bool)))
    else:
        for c in build_out:
            ok = bi >= 0
            idx = np.where(ok, bi, 0)
            cols.append((bcols[c][idx], ~ok | bmasks[c][idx]))
    return [(v[inner], m[inner]) for v, m in cols], [(v[~inner], m[~inner]) for v, m in cols]


CASES = [("LEFT", "UNKNOWN"), ("RIGHT", "UNKNOWN"), ("LEFT", "LEFT"), ("RIGHT", "RIGHT"), ("FULL", "UNKNOWN"),
         ("LEFT_SEMI", "UNKNOWN"), ("LEFT_ANTI", "UNKNOWN"), ("EXISTENCE", "UNKNOWN"), ("INNER", "LEFT")]


@pytest.mark.parametrize("join_type,build_side", CASES)
@pytest.mark.parametrize("dense,dup", [(True, False), (False, True)])
def test_join_types_match_oracle(join_type, build_side, dense, dup):
    """Random builds (ARRAY table with unique keys, HASH table with duplicate keys; NULL keys
    and payloads) probed in ragged batches, every output row checked against the oracle."""
    n_build, n_probe = 60_000, 250_000
    seed = 2 * CASES.index((join_type, build_side)) + int(dense)
    bcols, bmasks, pcols, pmasks = _random_join_input(n_build, n_probe, dense, dup, seed)
    kind = oracle.join_kind(join_type, build_side)
    probe_out = [0, 1]
    build_out = [] if kind in ("semi", "existence") else [2, 1]
    cols, outer, n_outer = run_typed_join(join_type, build_side, [L, I, L], bcols, bmasks, 0, [L, I], pcols, pmasks,
                                          0, probe_out, build_out, batch_sizes=(4096, 1000, 7777),
                                          build_batches=2, pipeline=dense)
    exp_probe, exp_outer = _expected_cols(kind, bcols, bmasks, pcols, pmasks, probe_out, build_out)
    got = rows_matrix(cols) if cols is not None else np.zeros((0, 0), np.int64)
    want = rows_matrix(exp_probe)
    assert got.shape[0] == want.shape[0]
    assert np.array_equal(got, want)
    if kind in ("build_outer", "full"):
        want_outer = rows_matrix(exp_outer)
        got_outer = rows_matrix(outer) if outer is not None else np.zeros((0, 0), np.int64)
        assert got_outer.shape[0] == want_outer.shape[0] > 0
        assert np.array_equal(got_outer, want_outer)
        row_bytes = 8 + 4 + 8 + 4
        assert n_outer == -(-want_outer.shape[0] // -(-(1 << 20) // row_bytes))


def test_outer_operator_with_build_left_lists_build_columns_first():
    k = JOIN_TYPED["left_join_build_left"]
    (b, bm), (p, pm) = kat_columns(k)
    _, outer, _ = run_typed_join("LEFT", "LEFT", [L, L], b, bm, 1, [L, L], p, pm, 1, [0, 1], [0, 1],
                                 outer_side=omg.OMNI_BUILD_LEFT)
    assert sorted(map(row_key, _rows(outer))) == sorted(map(row_key, k["outer_rows"]))


def test_full_join_without_probe_rows_emits_every_build_row():
    b = [np.arange(10, dtype=np.int64), np.arange(10, dtype=np.int64) * 3]
    bm = [np.zeros(10, bool), np.zeros(10, bool)]
    bm[0][4] = True
    cols, outer, n_outer = run_typed_join("FULL", "UNKNOWN", [L, L], b, bm, 0, [L], [np.zeros(0, np.int64)],
                                          [np.zeros(0, bool)], 0, [0], [1])
    assert cols is None and n_outer == 1
    assert sorted(map(row_key, _rows(outer))) == sorted(map(row_key, [[None, 3 * i] for i in range(10)]))


@pytest.mark.parametrize("join_type", ["INNER", "LEFT", "FULL", "LEFT_SEMI", "LEFT_ANTI", "EXISTENCE"])
@pytest.mark.parametrize("shape", ["int_long", "short_long_int", "decimal128"])
def test_multi_column_keys_match_oracle(join_type, shape):
    """Keys of several columns (and one 16-byte decimal key): the table holds the tuple hash and
    every candidate is compared column by column, so equal hashes of different tuples never
    match.  Duplicates, NULL key columns (any NULL: no match) and every output row checked."""
    rng = np.random.default_rng(["int_long", "short_long_int", "decimal128"].index(shape) * 10 + len(join_type))
    nb, npr = 40_000, 150_000
    pool = 12_000
    if shape == "int_long":
        kt = [I, L]
        dom = [rng.integers(-50, 50, pool).astype(np.int32), rng.integers(-2**40, 2**40, pool)]
    elif shape == "short_long_int":
        kt = [S, L, I]
        dom = [rng.integers(-3, 3, pool).astype(np.int16), rng.integers(0, 40, pool).astype(np.int64),
               rng.integers(-2**31, 2**31, pool, dtype=np.int64).astype(np.int32)]
    else:
        kt = [omg.Decimal128Type(38, 2)]
        lo = rng.integers(0, 2**63, pool, dtype=np.int64).astype(np.uint64)
        hi = rng.integers(-3, 3, pool).astype(np.int64).astype(np.uint64)
        dom = [np.stack([lo, hi], axis=1)]
    bsel = rng.integers(0, pool // 2, nb)
    psel = rng.integers(0, pool, npr)
    nk = len(kt)
    bkeys = [d[bsel] for d in dom]
    pkeys = [d[psel] for d in dom]
    bkm = [rng.random(nb) < 0.02 for _ in range(nk)]
    pkm = [rng.random(npr) < 0.02 for _ in range(nk)]
    bpay = rng.integers(-2**62, 2**62, nb)
    ppay = rng.integers(-2**31, 2**31, npr, dtype=np.int64).astype(np.int32)
    bcols, bmasks = bkeys + [bpay], bkm + [np.zeros(nb, bool)]
    pcols, pmasks = pkeys + [ppay], pkm + [rng.random(npr) < 0.05]
    kind = oracle.join_kind(join_type, "UNKNOWN")
    probe_out = list(range(nk + 1))
    build_out = [] if kind in ("semi", "existence", "anti") else [nk] + list(range(nk))
    cols, outer, _ = run_typed_join(join_type, "UNKNOWN", kt + [L], bcols, bmasks, list(range(nk)), kt + [I],
                                    pcols, pmasks, list(range(nk)), probe_out, build_out, batch_sizes=(4096, 5000))
    bid, bn, pid, pn = tuple_ids(bkeys, bkm, pkeys, pkm)
    pi_all, bi_all = oracle.join(kind, bid, bn, pid, pn)

    def flat(values, masks, idx, cols_):
        out = []
        ok = idx >= 0
        j = np.where(ok, idx, 0)
        for c in cols_:
            v, m = values[c], masks[c]
            if v.ndim == 2:  # decimal128: compare both words
                out += [(v[j, 0].astype(np.int64), ~ok | m[j]), (v[j, 1].astype(np.int64), ~ok | m[j])]
            else:
                out.append((v[j], ~ok | m[j]))
        return out
    def split_words(cols_):
        out = []
        for v, m in (cols_ or []):
            if v.ndim == 2:
                out += [(v[:, 0].astype(np.int64), m), (v[:, 1].astype(np.int64), m)]
            else:
                out.append((v, m))
        return out

    # Probe-operator rows, then (full joins) the outer-join operator's unmatched build rows.
    for part, got_cols in (("probe", cols), ("outer", outer)):
        sel = (pi_all >= 0) if part == "probe" else (pi_all < 0)
        if part == "outer" and kind != "full":
            assert outer is None
            continue
        pi, bi = pi_all[sel], bi_all[sel]
        want = flat(pcols, pmasks, pi, probe_out)
        want += [(bi, np.zeros(len(bi), bool))] if kind == "existence" else flat(bcols, bmasks, bi, build_out)
        got = split_words(got_cols)
        got_m = rows_matrix(got) if got else np.zeros((0, 0), np.int64)
        want_m = rows_matrix(want)
        assert got_m.shape[0] == want_m.shape[0] and len(pi) > 0, part
        assert np.array_equal(got_m, want_m), part


@pytest.mark.parametrize("join_type,build_side", CASES)
def test_bitmap_probe_every_kind_matches_oracle(join_type, build_side):
    """A unique ARRAY build (NULL-free build output: the packed slot payload) probed in one large
    batch: the bitmap kernel takes every join kind, marking matched build rows visited through
    the slot's entry for the kinds that keep unmatched build rows; probe-side and outer-join rows
    against the oracle."""
    n_build, n_probe = 60_000, 400_000
    bcols, bmasks, pcols, pmasks = _random_join_input(n_build, n_probe, True, False, 77 + CASES.index(
        (join_type, build_side)))
    kind = oracle.join_kind(join_type, build_side)
    probe_out = [0, 1]
    build_out = [] if kind in ("semi", "existence") else [2]
    cols, outer, _ = run_typed_join(join_type, build_side, [L, I, L], bcols, bmasks, 0, [L, I], pcols, pmasks,
                                    0, probe_out, build_out, batch_sizes=(n_probe,))
    assert omg.lib().omg_debug_last_probe_kernel() == 4
    exp_probe, exp_outer = _expected_cols(kind, bcols, bmasks, pcols, pmasks, probe_out, build_out)
    got = rows_matrix(cols) if cols is not None else np.zeros((0, 0), np.int64)
    want = rows_matrix(exp_probe)
    assert got.shape[0] == want.shape[0] > 0
    assert np.array_equal(got, want)
    if kind in ("build_outer", "full"):
        want_outer = rows_matrix(exp_outer)
        got_outer = rows_matrix(outer) if outer is not None else np.zeros((0, 0), np.int64)
        assert got_outer.shape[0] == want_outer.shape[0] > 0
        assert np.array_equal(got_outer, want_outer)
