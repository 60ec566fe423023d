"""Multi-column join keys of fixed widths packed into one 64-bit key (a mixed-radix number over
the build's per-column value ranges), checked against the oracle's join of the same key tuples.

The reference hashes and compares the key columns of a row together
(join_hash_table_variants.cpp:573-609); packing is exact for fixed-width columns whose build
ranges multiply to at most 2^62, and other keys keep the tuple-hash path."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import rows_matrix, split, tuple_ids

L, I, S = omg.LongType(), omg.IntType(), omg.ShortType()
pytestmark = pytest.mark.gpu

# omg_debug_last_probe_kernel codes
KIND_KERNEL, BITS_KERNEL = 1, 4


def _run(join_type, btypes, bcols, bmasks, nk, ptypes, pcols, pmasks, probe_out, build_out, batch_sizes,
         device=False, pipeline=True):
    jt = oracle.JOIN_TYPES[join_type]
    bf = omg.HashBuilderOperatorFactory(jt, btypes, list(range(nk)))
    bop = bf.create_operator()
    bop.add_input(omg.make_batch(btypes, bcols, bmasks))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory(ptypes, probe_out, list(range(nk)), build_out, [btypes[c] for c in build_out],
                                       bf)
    pop = pf.create_operator()
    if pipeline:
        pop.set_no_more_input(False)
    outs = []
    for s, e in split(len(pcols[0]), list(batch_sizes)):
        b = omg.make_batch(ptypes, [c[s:e] for c in pcols], [m[s:e] for m in pmasks])
        if device:
            d = omg.batch_to_device(b)
            omg.free_batch(b)
            b = d
        pop.add_input(b)
        if not pipeline:
            outs += pop.drain()
    if pipeline:
        outs += pop.drain()
        pop.no_more_input()
        outs += pop.drain()
    kernel = omg.lib().omg_debug_last_probe_kernel()
    cols = None
    for b in outs:
        if device:
            h = omg.batch_to_host(b)
            omg.free_batch(b)
            b = h
        c = omg.batch_to_numpy(b)
        omg.free_batch(b)
        cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                       for a, x in zip(cols, c)]
    pop.delete()
    pf.close()
    bop.delete()
    bf.close()
    return cols, kernel


def _expected(kind, bcols, bmasks, pcols, pmasks, nk, probe_out, build_out):
    bid, bn, pid, pn = tuple_ids(bcols[:nk], bmasks[:nk], pcols[:nk], pmasks[:nk])
    pi, bi = oracle.join(kind, bid, bn, pid, pn)
    sel = pi >= 0
    pi, bi = pi[sel], bi[sel]
    out = [(pcols[c][pi], pmasks[c][pi]) for c in probe_out]
    ok = bi >= 0
    j = np.where(ok, bi, 0)
    out += [(bcols[c][j], ~ok | bmasks[c][j]) for c in build_out]
    return out


def _check(join_type, btypes, bcols, bmasks, nk, ptypes, pcols, pmasks, probe_out, build_out, batch_sizes=(1 << 20,),
           device=False):
    kind = oracle.join_kind(join_type, "UNKNOWN")
    got, kernel = _run(join_type, btypes, bcols, bmasks, nk, ptypes, pcols, pmasks, probe_out, build_out, batch_sizes,
                       device=device)
    want = _expected(kind, bcols, bmasks, pcols, pmasks, nk, probe_out, build_out)
    g = rows_matrix(got) if got else np.zeros((0, 0), np.int64)
    w = rows_matrix(want)
    assert g.shape == w.shape and w.shape[0] > 0
    assert np.array_equal(g, w)
    return kernel


def _hi_lo(n_build, n_probe, seed):
    """The headline join's keys split into (key >> 10, key & 1023) int32 pairs: the packed key is
    dense, so the table is an ARRAY table probed by the bitmap kernel."""
    rng = np.random.default_rng(seed)
    bkey = rng.permutation(n_build).astype(np.int64)
    match = rng.random(n_probe) < 0.8
    pkey = np.where(match, bkey[rng.integers(0, n_build, n_probe)], rng.integers(n_build, 2 * n_build, n_probe))
    bcols = [(bkey >> 10).astype(np.int32), (bkey & 1023).astype(np.int32),
             rng.integers(-2**31, 2**31, n_build, dtype=np.int64).astype(np.int32),
             rng.integers(-2**31, 2**31, n_build, dtype=np.int64).astype(np.int32)]
    pcols = [(pkey >> 10).astype(np.int32), (pkey & 1023).astype(np.int32)]
    bmasks = [np.zeros(n_build, bool) for _ in bcols]
    pmasks = [rng.random(n_probe) < 0.01, rng.random(n_probe) < 0.01]
    return bcols, bmasks, pcols, pmasks


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("batch", [1 << 20, 4096, 3000])
def test_two_int32_key_columns_take_the_bitmap_probe(gpu, device, batch):
    bcols, bmasks, pcols, pmasks = _hi_lo(1 << 16, 500_000, 51)
    kernel = _check("INNER", [I, I, I, I], bcols, bmasks, 2, [I, I], pcols, pmasks, [0, 1], [2, 3],
                    batch_sizes=(batch,), device=device)
    assert kernel == BITS_KERNEL


@pytest.mark.parametrize("join_type", ["INNER", "LEFT", "LEFT_SEMI", "LEFT_ANTI", "EXISTENCE", "FULL"])
def test_packed_keys_with_nulls_and_out_of_range_parts(gpu, join_type):
    """(SHORT, LONG, INT) keys with NULL parts on both sides, negative values, duplicates in the
    build, and probe parts below and above every build range."""
    rng = np.random.default_rng(52 + len(join_type))
    nb, npr = 30_000, 200_000
    b0 = rng.integers(-40, 40, nb).astype(np.int16)
    b1 = rng.integers(-10**9, 10**9, nb)
    b2 = rng.integers(-500, 500, nb).astype(np.int32)
    pick = rng.integers(0, nb, npr)
    p0 = np.where(rng.random(npr) < 0.1, rng.integers(-100, 100, npr), b0[pick]).astype(np.int16)
    p1 = np.where(rng.random(npr) < 0.1, rng.integers(-2 * 10**9, 2 * 10**9, npr), b1[pick])
    p2 = np.where(rng.random(npr) < 0.1, rng.integers(-2000, 2000, npr), b2[pick]).astype(np.int32)
    bpay = rng.integers(-2**62, 2**62, nb)
    ppay = rng.integers(-2**31, 2**31, npr, dtype=np.int64).astype(np.int32)
    bcols = [b0, b1, b2, bpay]
    bmasks = [rng.random(nb) < 0.02 for _ in range(3)] + [rng.random(nb) < 0.05]
    pcols = [p0, p1, p2, ppay]
    pmasks = [rng.random(npr) < 0.02 for _ in range(3)] + [rng.random(npr) < 0.05]
    kind = oracle.join_kind(join_type, "UNKNOWN")
    build_out = [] if kind in ("semi", "anti", "existence") else [3, 0]
    if join_type == "FULL":
        # Probe-side rows only (the outer operator's build rows are covered by the join-type tests).
        got, _ = _run(join_type, [S, L, I, L], bcols, bmasks, 3, [S, L, I, I], pcols, pmasks, [0, 1, 2, 3], build_out,
                      (4096, 5000))
        want = _expected("probe_outer", bcols, bmasks, pcols, pmasks, 3, [0, 1, 2, 3], build_out)
        assert np.array_equal(rows_matrix(got), rows_matrix(want))
        return
    if kind == "existence":
        got, _ = _run(join_type, [S, L, I, L], bcols, bmasks, 3, [S, L, I, I], pcols, pmasks, [0, 3], [], (4096, 5000))
        bid, bn, pid, pn = tuple_ids(bcols[:3], bmasks[:3], pcols[:3], pmasks[:3])
        pi, bi = oracle.join(kind, bid, bn, pid, pn)
        want = [(pcols[0][pi], pmasks[0][pi]), (pcols[3][pi], pmasks[3][pi]), (bi, np.zeros(len(bi), bool))]
        assert np.array_equal(rows_matrix(got), rows_matrix(want))
        return
    _check(join_type, [S, L, I, L], bcols, bmasks, 3, [S, L, I, I], pcols, pmasks, [0, 1, 2, 3], build_out,
           batch_sizes=(4096, 5000))


def test_keys_too_wide_to_pack_keep_the_tuple_hash(gpu):
    """Two LONG key columns over their full range: the ranges multiply past 2^62, so the table
    holds tuple hashes and the probe compares columns (the multi-key kernel)."""
    rng = np.random.default_rng(53)
    nb, npr = 20_000, 100_000
    b0 = rng.integers(-2**62, 2**62, nb)
    b1 = rng.integers(-2**62, 2**62, nb)
    pick = rng.integers(0, nb, npr)
    p0 = np.where(rng.random(npr) < 0.3, rng.integers(-2**62, 2**62, npr), b0[pick])
    p1 = b1[pick]
    bpay = rng.integers(0, 1000, nb)
    bcols, bmasks = [b0, b1, bpay], [np.zeros(nb, bool)] * 3
    pcols, pmasks = [p0, p1], [rng.random(npr) < 0.01, np.zeros(npr, bool)]
    kernel = _check("INNER", [L, L, L], bcols, bmasks, 2, [L, L], pcols, pmasks, [0, 1], [2],
                    batch_sizes=(4096, 3000))
    assert kernel == KIND_KERNEL
