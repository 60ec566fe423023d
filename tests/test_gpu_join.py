"""GPU parity of HashBuilder + LookupJoin (inner) against the oracle: the output row multiset must
equal the oracle's exactly, NULLs included."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import expected_join_rows, join_rows_canonical, run_join

pytestmark = pytest.mark.gpu

L, I, S = omg.LongType(), omg.IntType(), omg.ShortType()


def _cfg2_like(nb, npb, seed, dup=False, sparse=False):
    rng = np.random.default_rng(seed)
    if sparse:
        bkey = (rng.choice(2**39, nb, replace=False) * 2).astype(np.int64)
    else:
        bkey = rng.permutation(nb).astype(np.int64)
    if dup:
        bkey = np.concatenate([bkey, bkey[: nb // 3], bkey[: nb // 10]])
    p1 = rng.integers(-2**31, 2**31, len(bkey), dtype=np.int64).astype(np.int32)
    p2 = rng.integers(-2**31, 2**31, len(bkey), dtype=np.int64).astype(np.int32)
    match = rng.random(npb) < 0.8
    if sparse:
        miss = (rng.integers(0, 2**39, npb) * 2 + 1).astype(np.int64)
    else:
        miss = rng.integers(nb, 2 * nb, npb).astype(np.int64)
    pkey = np.where(match, bkey[rng.integers(0, nb, npb)], miss)
    pnull = rng.random(npb) < 0.01
    return bkey, p1, p2, pkey, pnull


def _check(bkey, p1, p2, pkey, pnull, bnulls=None, **kw):
    bcols = [bkey, p1, p2]
    got, max_rows = run_join([L, I, I], bcols, bnulls, [0], [L], [pkey], [pnull], [0], [0], [1, 2], **kw)
    exp = expected_join_rows([pkey], [pnull], bcols, bnulls, 0, 0, [0], [1, 2])
    assert join_rows_canonical(got) == exp
    # 16-byte rows: at most ceil(1 MiB / 16) = 65536 rows per output batch (lookup_join.cpp:1628-1640)
    assert max_rows <= 65536
    return got


def test_config2_shape_array_table(gpu):
    _check(*_cfg2_like(50_000, 400_000, 1))


def test_config2_shape_pipeline_mode(gpu):
    _check(*_cfg2_like(50_000, 300_000, 2), pipeline=True, batch_sizes=(4096, 100, 3000))


def test_device_resident_probe(gpu):
    _check(*_cfg2_like(20_000, 200_000, 3), device_input=True, batch_sizes=(200_000,))


def test_bitmap_probe_large_device_batch(gpu):
    # >= 64 tiles on an ARRAY table with a packed payload: the shared-memory bitmap kernel,
    # output spread over 16 regions.
    _check(*_cfg2_like(100_000, 1_200_000, 11), device_input=True, batch_sizes=(1_200_000,))


def test_bitmap_probe_negative_key_range(gpu):
    bkey, p1, p2, pkey, pnull = _cfg2_like(60_000, 700_000, 12)
    _check(bkey - 30_000, p1, p2, pkey - 30_000, pnull, pipeline=True, batch_sizes=(4096, 1000, 64))


def test_regions_with_duplicates_retry(gpu):
    # Duplicate build keys: region capacities start at 2x their probe rows and are re-sized
    # from the exact per-region counts when exceeded.
    bkey, p1, p2, pkey, pnull = _cfg2_like(20_000, 500_000, 13, dup=True)
    hot = bkey[:50]
    bkey = np.concatenate([bkey] + [hot] * 6)
    p1 = np.concatenate([p1, np.tile(p1[:50], 6)])
    p2 = np.concatenate([p2, np.tile(p2[:50], 6)])
    pkey = np.where(np.arange(len(pkey)) % 3 == 0, hot[np.arange(len(pkey)) % 50], pkey)
    _check(bkey, p1, p2, pkey, pnull, pipeline=True, batch_sizes=(4096,))


def test_duplicate_build_keys_array_mode(gpu):
    _check(*_cfg2_like(30_000, 200_000, 4, dup=True))


def test_sparse_keys_hash_mode(gpu):
    _check(*_cfg2_like(40_000, 200_000, 5, sparse=True))


def test_sparse_keys_hash_mode_duplicates(gpu):
    _check(*_cfg2_like(40_000, 200_000, 6, sparse=True, dup=True))


def test_nulls_in_build_keys_and_payloads(gpu):
    bkey, p1, p2, pkey, pnull = _cfg2_like(20_000, 100_000, 7)
    rng = np.random.default_rng(70)
    bn = [rng.random(len(bkey)) < 0.05, rng.random(len(bkey)) < 0.1, None]
    _check(bkey, p1, p2, pkey, pnull, bnulls=bn)


def test_extreme_keys_including_int64_min(gpu):
    mn, mx = np.iinfo(np.int64).min, np.iinfo(np.int64).max
    bkey = np.array([mn, mx, 0, -1, mn, 5], dtype=np.int64)
    p1 = np.arange(6, dtype=np.int32)
    p2 = -np.arange(6, dtype=np.int32)
    pkey = np.array([mn, mx, 0, 7, -1, mn, 5, 5], dtype=np.int64)
    pnull = np.array([0, 0, 0, 0, 0, 0, 1, 0], dtype=bool)
    _check(bkey, p1, p2, pkey, pnull)


def test_probe_payload_columns_and_narrow_keys(gpu):
    rng = np.random.default_rng(8)
    nb, npb = 5000, 60_000
    bkey = rng.integers(-20000, 20000, nb).astype(np.int32)
    bval = rng.integers(0, 100, nb).astype(np.int16)
    pkey = rng.integers(-20000, 20000, npb).astype(np.int32)
    pval = rng.standard_normal(npb)
    pvn = rng.random(npb) < 0.05
    D = omg.DoubleType()
    got, _ = run_join([I, S], [bkey, bval], None, [0], [D, I], [pval, pkey], [pvn, None], [1], [1, 0], [1, 0])
    exp = expected_join_rows([pval, pkey], [pvn, None], [bkey, bval], None, 1, 0, [1, 0], [1, 0])
    assert join_rows_canonical(got) == exp


def test_empty_build_and_no_matches(gpu):
    bkey = np.zeros(0, dtype=np.int64)
    p = np.zeros(0, dtype=np.int32)
    pkey = np.arange(100, dtype=np.int64)
    got, _ = run_join([L, I, I], [bkey, p, p], None, [0], [L], [pkey], None, [0], [0], [1, 2])
    assert got is None
    bkey = np.arange(100, 200, dtype=np.int64)
    p = np.arange(100, dtype=np.int32)
    got, _ = run_join([L, I, I], [bkey, p, p], None, [0], [L], [pkey], None, [0], [0], [1, 2])
    assert got is None


def test_reference_kat_inner_join_one_build_op(gpu):
    """join_test.cpp:52-109,283-305 (TestInnerEqualityJoinWithOneBuildOp)."""
    import json
    from pathlib import Path

    g = json.loads((Path(__file__).parent / "golden" / "join_kats.json").read_text())["inner_join_one_build_op"]
    got, _ = run_join([L, L], [np.array(g["build"][0], np.int64), np.array(g["build"][1], np.int64)], None, [0],
                      [L, L], [np.array(g["probe"][0], np.int64), np.array(g["probe"][1], np.int64)], None, [0],
                      [1], [1])
    exp = sorted(tuple(r) for r in g["expected_rows"])
    assert join_rows_canonical(got) == exp


def test_reference_kat_array_table_short_keys(gpu):
    """join_test.cpp:4265-4313 (TestInnerEqualityJoinOfArrayTable)."""
    import json
    from pathlib import Path

    g = json.loads((Path(__file__).parent / "golden" / "join_kats.json").read_text())["array_table_short"]
    got, _ = run_join([S, S], [np.array(c, np.int16) for c in g["build"]], None, [0], [S, S],
                      [np.array(c, np.int16) for c in g["probe"]], None, [0], [0, 1], [0, 1])
    exp = sorted(tuple(r) for r in g["expected_rows"])
    assert join_rows_canonical(got) == exp


def test_bulk_add_inputs_and_get_outputs(gpu):
    """omg_op_add_inputs / omg_op_get_outputs equal the per-batch AddInput / GetOutput calls."""
    bkey, p1, p2, pkey, pnull = _cfg2_like(30_000, 300_000, 14)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I, I], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, I, I], [bkey, p1, p2]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf)
    op = pf.create_operator()
    op.set_no_more_input(False)
    batches = [omg.make_batch([L], [pkey[s:s + 4096]], [pnull[s:s + 4096]]) for s in range(0, len(pkey), 4096)]
    op.add_inputs(batches[:40])
    outs, rows = op.get_outputs(1 << 12)
    op.add_inputs(batches[40:])
    op.no_more_input()
    more, rows2 = op.get_outputs(1 << 12)
    outs += more
    assert op.get_status() == omg.OMNI_STATUS_FINISHED
    per = [omg.batch_to_numpy(b) for b in outs]
    cols = [(np.concatenate([p[c][0] for p in per]), np.concatenate([p[c][1] for p in per])) for c in range(3)]
    assert rows + rows2 == len(cols[0][0])
    omg.free_batches(outs)
    op.delete()
    pf.close()
    bop.delete()
    bf.close()
    exp = expected_join_rows([pkey], [pnull], [bkey, p1, p2], None, 0, 0, [0], [1, 2])
    assert join_rows_canonical(cols) == exp


@pytest.mark.parametrize("join_type", [omg.OMNI_JOIN_TYPE_INNER, omg.OMNI_JOIN_TYPE_LEFT])
def test_pipelined_probe_chunks_in_flight(gpu, join_type):
    """Pipelined callers: every full 2^22-row chunk of queued batches is launched by AddInput and
    finished by a later GetOutput (up to two in flight), outputs written straight to host memory.
    Three and a half chunks of probe rows give the same row multiset as the oracle."""
    rng = np.random.default_rng(21 + join_type)
    nb = 1 << 16
    bkey = rng.permutation(nb).astype(np.int64)
    p1 = rng.integers(-1000, 1000, nb).astype(np.int32)
    p2 = rng.integers(-1000, 1000, nb).astype(np.int32)
    n = 7 << 21
    pkey = rng.integers(0, nb + nb // 4, n).astype(np.int64)
    pnull = rng.random(n) < 0.01
    bf = omg.HashBuilderOperatorFactory(join_type, [L, I, I], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, I, I], [bkey, p1, p2]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf)
    op = pf.create_operator()
    op.set_no_more_input(False)
    cols = [[], [], []]
    masks = [[], [], []]

    def take(outs):
        for b in outs:
            for c, (v, m) in enumerate(omg.batch_to_numpy(b)):
                cols[c].append(v)
                masks[c].append(m)
        omg.free_batches(outs)

    step = 1024 * 4096
    for s in range(0, n, step):
        batches = [omg.make_batch([L], [pkey[i:i + 4096]], [pnull[i:i + 4096]])
                   for i in range(s, min(n, s + step), 4096)]
        op.add_inputs(batches)
        take(op.get_outputs(1 << 12)[0])
    op.no_more_input()
    take(op.get_outputs(1 << 12)[0])
    assert op.get_status() == omg.OMNI_STATUS_FINISHED
    op.delete()
    pf.close()
    bop.delete()
    bf.close()
    got = [np.concatenate(c) for c in cols]
    gm = [np.concatenate(m) for m in masks]
    kind = "inner" if join_type == omg.OMNI_JOIN_TYPE_INNER else "probe_outer"
    pi, bi = oracle.join(kind, bkey, None, pkey, pnull)
    want_k = np.where(pnull[pi], 0, pkey[pi])
    want_p1 = np.where(bi >= 0, p1[np.maximum(bi, 0)], 0)
    want_p2 = np.where(bi >= 0, p2[np.maximum(bi, 0)], 0)
    want_m = [pnull[pi], bi < 0, bi < 0]
    got_rows = np.stack([np.where(gm[0], 0, got[0]), gm[0], np.where(gm[1], 0, got[1]), gm[1],
                         np.where(gm[2], 0, got[2]), gm[2]]).astype(np.int64)
    want_rows = np.stack([want_k, want_m[0], want_p1, want_m[1], want_p2, want_m[2]]).astype(np.int64)
    assert got_rows.shape == want_rows.shape
    g_sorted = got_rows[:, np.lexsort(got_rows[::-1])]
    w_sorted = want_rows[:, np.lexsort(want_rows[::-1])]
    assert np.array_equal(g_sorted, w_sorted)


@pytest.mark.parametrize("device_input", [False, True])
@pytest.mark.parametrize("batch", [4096, 3000, 1 << 20])
def test_staged_and_per_warp_probe_kernels_agree(gpu, device_input, batch):
    """The group-staged inner probe (whole-line output runs) and the per-warp bitmap probe give
    the oracle's rows, for one large batch and for many ragged batches, host and HBM input."""
    bkey, p1, p2, pkey, pnull = _cfg2_like(1 << 16, 600_000, 41)
    try:
        for staged in (1, 0):
            omg.lib().omg_debug_set_staged_probe(staged)
            _check(bkey, p1, p2, pkey, pnull, batch_sizes=(batch,), device_input=device_input)
    finally:
        omg.lib().omg_debug_set_staged_probe(1)


@pytest.mark.parametrize("bulk", [1, 2, 0])
@pytest.mark.parametrize("batch", [1 << 20, 4096, 3000, 1000])
def test_bulk_copy_probe_kernel_hbm_output(gpu, bulk, batch):
    """Device input and HBM output: the bulk-copy probe (keys staged into shared memory by
    cp.async.bulk; mode 2 also stores the output runs back by cp.async.bulk) and the per-lane
    bitmap probe (mode 0) give the expected rows, for one large batch, whole tiles and ragged
    batches (partial segments read their keys with plain loads)."""
    bkey, p1, p2, pkey, pnull = _cfg2_like(1 << 16, 700_000, 43)
    try:
        assert omg.lib().omg_debug_set_bulk_probe(bulk) == 0
        _check(bkey, p1, p2, pkey, pnull, batch_sizes=(batch,), device_input=True, device_output=True,
               pipeline=True)
        assert omg.lib().omg_debug_last_probe_kernel() == (6 if bulk else 4)
    finally:
        omg.lib().omg_debug_set_bulk_probe(0)


@pytest.mark.parametrize("bulk", [1, 2])
def test_bulk_copy_probe_two_payload_layouts(gpu, bulk):
    """The (8-byte key, 8-byte payload) and (8-byte key, 4-byte payload) layouts of the
    bulk-copy probe, no NULL keys, against the expected rows."""
    rng = np.random.default_rng(44)
    nb, n = 1 << 16, 600_000
    bkey = rng.permutation(nb).astype(np.int64)
    pay8 = rng.integers(-2**62, 2**62, nb, dtype=np.int64)
    pay4 = rng.integers(-2**31, 2**31, nb, dtype=np.int64).astype(np.int32)
    pkey = rng.integers(0, 2 * nb, n).astype(np.int64)
    try:
        assert omg.lib().omg_debug_set_bulk_probe(bulk) == 0
        for btypes, bcols in (([L, L], [bkey, pay8]), ([L, I], [bkey, pay4])):
            got, _ = run_join(btypes, bcols, None, [0], [L], [pkey], None, [0], [0], [1],
                              batch_sizes=(n,), device_input=True, device_output=True)
            exp = expected_join_rows([pkey], None, bcols, None, 0, 0, [0], [1])
            assert join_rows_canonical(got) == exp
            assert omg.lib().omg_debug_last_probe_kernel() == 6
    finally:
        omg.lib().omg_debug_set_bulk_probe(0)


def test_bulk_probe_knob_rejects_other_modes():
    assert omg.lib().omg_debug_set_bulk_probe(3) != 0
    assert omg.lib().omg_debug_set_bulk_probe(0) == 0


@pytest.mark.parametrize("device_input,device_output", [(False, False), (True, False), (True, True)])
def test_worker_pipeline_matches_oracle(gpu, device_input, device_output):
    """Pipelined callers (SetNoMoreInput(false)) hand full chunks to the operator's worker
    thread, which launches and finishes the probe calls while the caller keeps adding batches:
    small chunks (40,000 rows) so that many chunks run, ragged batches, against the oracle."""
    bkey, p1, p2, pkey, pnull = _cfg2_like(1 << 16, 700_000, 45)
    try:
        omg.lib().omg_debug_set_probe_chunk_rows(40_000)
        _check(bkey, p1, p2, pkey, pnull, batch_sizes=(4096, 777, 10_000), pipeline=True,
               device_input=device_input, device_output=device_output)
    finally:
        omg.lib().omg_debug_set_probe_chunk_rows(0)


def test_worker_pipeline_error_reaches_the_caller(gpu):
    """An allocation failure inside the worker thread (host-side fault injection) comes back to
    the caller as OMG_ERR_OOM from a later AddInput or GetOutput, and the operator is deleted
    cleanly afterwards."""
    bkey, p1, p2, pkey, pnull = _cfg2_like(1 << 14, 200_000, 46)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I, I], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, I, I], [bkey, p1, p2]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf)
    pop = pf.create_operator()
    batches = [omg.make_batch([L], [pkey[s:s + 4096]], [pnull[s:s + 4096]]) for s in range(0, len(pkey), 4096)]
    errors = []
    try:
        omg.lib().omg_debug_set_probe_chunk_rows(20_000)
        pop.set_no_more_input(False)
        omg.lib().omg_debug_fail_next_allocs(1000)
        for i, b in enumerate(batches):
            try:
                pop.add_input(b)
            except omg.OmgError as e:
                errors.append(e.status)
        pop.no_more_input()
        try:
            pop.drain()
        except omg.OmgError as e:
            errors.append(e.status)
    finally:
        omg.lib().omg_debug_fail_next_allocs(0)
        omg.lib().omg_debug_set_probe_chunk_rows(0)
    assert errors and all(s == -4 for s in errors), errors  # OMG_ERR_OOM
    pop.delete()
    pf.close()
    bop.delete()
    bf.close()
