"""Host-thread and bounded-wait behaviour on the GPU.

* Several probe operators of one LookupJoin factory run from several host threads against one
  shared build (the reference runs one probe operator per thread on a shared table,
  join/hash_builder.h:44-45, join_hash_table_variants.h:259-260); every thread's rows equal the
  oracle's inner join.
* A device-side wait for another thread's slot publication that runs out of its budget makes
  the call return OMG_ERR_TIMEOUT instead of hanging, and the context stays usable."""
import threading

import numpy as np
import pytest

import omnioperator_gb300 as omg
import oracle
from helpers import assert_agg_equal, join_rows_canonical, run_agg

pytestmark = pytest.mark.gpu

L, I = omg.LongType(), omg.IntType()


def test_probe_operators_on_host_threads_share_one_build(gpu):
    rng = np.random.default_rng(31)
    nb = 50_000
    bkey = rng.permutation(2 * nb)[:nb].astype(np.int64)
    bnull = rng.random(nb) < 0.01
    p1 = rng.integers(-2**31, 2**31, nb).astype(np.int32)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I], [0])
    bop = bf.create_operator()
    bop.add_input(omg.make_batch([L, I], [bkey, p1], [bnull, None]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1], [I], bf)
    n_threads, n_probe = 6, 120_000
    probes = []
    for t in range(n_threads):
        r = np.random.default_rng(100 + t)
        pk = np.where(r.random(n_probe) < 0.7, bkey[r.integers(0, nb, n_probe)], r.integers(2 * nb, 3 * nb, n_probe))
        probes.append((pk.astype(np.int64), r.random(n_probe) < 0.02))
    results, errors = [None] * n_threads, []
    start = threading.Barrier(n_threads)

    def work(t):
        try:
            op = pf.create_operator()
            pk, pn = probes[t]
            start.wait()
            outs = []
            for s in range(0, n_probe, 4096):
                op.add_input(omg.make_batch([L], [pk[s:s + 4096]], [pn[s:s + 4096]]))
                outs.extend(op.drain())
            cols = None
            for b in outs:
                c = omg.batch_to_numpy(b)
                omg.free_batch(b)
                cols = c if cols is None else [(np.concatenate([a[0], x[0]]), np.concatenate([a[1], x[1]]))
                                               for a, x in zip(cols, c)]
            op.delete()
            results[t] = cols
        except Exception as e:  # reported after the join
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(n_threads)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    pf.close()
    bop.delete()
    bf.close()
    assert not errors, errors
    for t in range(n_threads):
        pk, pn = probes[t]
        pi, bi = oracle.join_inner(bkey, bnull, pk, pn)
        want = sorted(zip(pk[pi].tolist(), p1[bi].tolist()))
        assert join_rows_canonical(results[t]) == want


def test_run_out_wait_budget_returns_timeout_not_a_hang(gpu):
    """Two-column keys go through the tag-published global table, where a thread that meets a
    slot being written waits for its publication.  With a one-tick budget such a wait gives up:
    the call either finishes (no thread had to wait) with the oracle's result, or returns
    OMG_ERR_TIMEOUT.  Afterwards, with the default budget, the same aggregation is correct."""
    rng = np.random.default_rng(5)
    n = 400_000
    k1 = rng.integers(0, 8, n).astype(np.int64)
    k2 = rng.integers(0, 4, n).astype(np.int32)
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    args = dict(group_cols=[0, 1], group_types=[L, I], aggs_cols=[[2]], agg_in_types=[[L]], agg_out_types=[[L]],
                funcs=[omg.OMNI_AGGREGATION_TYPE_SUM], columns=[k1, k2, v], types=[L, I, L],
                strategy=omg.AGG_STRATEGY_GLOBAL, batch_sizes=(1 << 17,))
    ora = oracle.hashagg([k1, k2], [oracle.T_LONG, oracle.T_INT], [None, None],
                         [dict(func=oracle.F_SUM, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)])
    outcomes = set()
    omg.lib().omg_debug_set_wait_budget(1)
    try:
        for _ in range(3):
            try:
                cols, _ = run_agg(**args)
                assert_agg_equal(cols, ora, 2)
                outcomes.add("ok")
            except omg.OmgError as e:
                assert e.status == -7, e
                outcomes.add("timeout")
    finally:
        omg.lib().omg_debug_set_wait_budget(0)
    assert outcomes
    cols, _ = run_agg(**args)
    assert_agg_equal(cols, ora, 2)
