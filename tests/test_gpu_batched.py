"""Batched aggregation (many tasks, one persistent launch, CUDA graph, autotuned shape) against
the oracle task by task: every task's output must equal a separate HashAggregation of that task
(bit-exact integers, doubles within the stated tolerance), including tasks re-run through the
exact path when their table overflows."""
import numpy as np
import pytest

import omnioperator_gb300 as omg
import omnioperator_gb300.sizer as sz
from helpers import assert_agg_equal, exact_by_key
from test_gpu_agg import _cfg1_aggs, _cfg1_oracle

pytestmark = pytest.mark.gpu

L, D = omg.LongType(), omg.DoubleType()


def _tasks(seed, n_tasks, max_rows=60_000, nulls=False):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_tasks):
        n = int(np.exp(rng.uniform(0, np.log(max_rows))))
        d = int(np.exp(rng.uniform(np.log(2), np.log(max(3, n)))))
        uniq = rng.integers(-2**62, 2**62, d, dtype=np.int64)
        key = uniq[rng.integers(0, d, n)]
        v1 = rng.integers(-10**6, 10**6, n, dtype=np.int64)
        v2 = rng.random(n)
        km = rng.random(n) < 0.02 if nulls else None
        m1 = rng.random(n) < 0.05 if nulls else None
        m2 = rng.random(n) < 0.05 if nulls else None
        out.append((key, v1, v2, km, m1, m2))
    return out


def _run(tasks, flags=0, sizer=None, runs=1):
    fac = omg.HashAggregationOperatorFactory(**{k: v for k, v in zip(
        ["group_by_cols", "group_input_types", "aggs_cols", "agg_input_types", "agg_output_types", "agg_func_types"],
        _cfg1_aggs().values())})
    handles = [omg.make_batch([L, L, D], [k, a, b], [km, m1, m2]) for k, a, b, km, m1, m2 in tasks]
    batch = omg.AggBatch(fac, handles, sizer=sizer, flags=flags)
    results = []
    for _ in range(runs):
        batch.run()
        per = {}
        for t, b in batch.outputs():
            if flags & omg.BATCH_DEVICE_OUTPUT:
                h = omg.batch_to_host(b)
                omg.free_batch(b)
                b = h
            per.setdefault(t, []).append(omg.batch_to_numpy(b))
            omg.free_batch(b)
        results.append(per)
    info = batch.info()
    batch.close()
    omg.free_batches(handles)
    fac.close()
    return results, info


def _check(tasks, per):
    for t, (key, v1, v2, km, m1, m2) in enumerate(tasks):
        parts = per.get(t, [])
        cols = [(np.concatenate([p[c][0] for p in parts]), np.concatenate([p[c][1] for p in parts]))
                for c in range(7)] if parts else None
        ora = _cfg1_oracle(key, km, v1, m1, v2, m2)
        valid = None if m2 is None else ~m2
        ex_sum = exact_by_key([key], [km], v2, valid)
        ex_avg = exact_by_key([key], [km], v2, valid, divide_by_count=True)
        assert_agg_equal(cols, ora, 1, double_aggs=(4, 5), exact={4: ex_sum, 5: ex_avg})


def test_batched_equals_separate_aggregations(gpu):
    tasks = _tasks(1, 120, nulls=True)
    (per,), info = _run(tasks)
    _check(tasks, per)
    # plain sizing may undersize a few tables; those tasks take the exact re-run path
    assert info["tasks"] == 120 and info["graph"] == 1 and info["reruns"] <= 12
    assert info["threads"] in (128, 256, 512, 1024)


def test_batched_graph_replays_give_the_same_result(gpu):
    tasks = _tasks(2, 60)
    (first, second), info = _run(tasks, runs=2)
    _check(tasks, first)
    _check(tasks, second)
    assert info["runs"] == 2 and info["graph"] == 1


def test_batched_overflowing_tasks_rerun_exactly(gpu):
    tasks = _tasks(3, 40, max_rows=20_000, nulls=True)
    (per,), info = _run(tasks, flags=omg.BATCH_DEBUG_TINY_TABLES)
    _check(tasks, per)
    assert info["reruns"] >= 5


@pytest.mark.parametrize("flags", [0, omg.BATCH_DEVICE_OUTPUT | omg.BATCH_NO_GRAPH])
def test_batched_grow_pass_finishes_overflowing_tasks(gpu, flags):
    """64-slot first tables: the tasks that outgrow them take one more batched run with tables of
    twice their rows (no operator re-runs), equal to the oracle task by task, over graph replays."""
    tasks = _tasks(5, 40, max_rows=20_000, nulls=True)
    (first, second), info = _run(tasks, flags=flags | omg.BATCH_DEBUG_TINY_GROW, runs=2)
    _check(tasks, first)
    _check(tasks, second)
    assert info["reruns"] >= 5 and info["grown"] == info["reruns"] and info["operator_reruns"] == 0


def test_batched_device_output_without_graph(gpu):
    tasks = _tasks(4, 50)
    (per,), info = _run(tasks, flags=omg.BATCH_DEVICE_OUTPUT | omg.BATCH_NO_GRAPH | omg.BATCH_NO_TUNE)
    _check(tasks, per)
    assert info["graph"] == 0


def test_batched_with_learned_sizer(gpu):
    model = sz.SizingModel.load(str(__import__("pathlib").Path(omg.__file__).parent / "models" / "agg_sizer.json"))
    tasks = _tasks(5, 80)
    (per,), info = _run(tasks, sizer=model)
    _check(tasks, per)
    assert info["learned"] == 1
    model.close()
