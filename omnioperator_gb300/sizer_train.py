"""Train the aggregation sizing model on records the plain operator logs.

    python -m omnioperator_gb300.sizer_train --out omnioperator_gb300/models/agg_sizer.json

Each training workload is a device-resident int64 key column generated on the GPU: N rows over
a domain of D values (a fraction of N), uniform or Zipf(s) by rank.  The plain operator
aggregates it (COUNT(*) by key) and logs its sizing record (the key sketch of its first flush)
and the group count it found; the network is then trained on those records by the library's
CUDA kernels and saved as JSON (dims + flat parameters).
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from . import api as omg
from . import sizer as sz


def zipf_cdf(torch, domain: int, s: float, dev):
    w = torch.arange(1, domain + 1, device=dev, dtype=torch.float64).pow_(-s)
    cdf = torch.cumsum(w, 0)
    cdf /= cdf[-1].clone()
    return cdf


def gpu_keys(torch, gen, n: int, domain: int, kind: str, s: float, salt: int, dev, cdf=None):
    """n int64 keys on the GPU: rank uniform or Zipf(s) over `domain`, mixed to 64 bits."""
    if kind == "uniform":
        r = torch.randint(0, domain, (n,), generator=gen, device=dev, dtype=torch.int64)
    else:
        if cdf is None:
            cdf = zipf_cdf(torch, domain, s, dev)
        u = torch.rand(n, generator=gen, device=dev, dtype=torch.float64)
        r = torch.searchsorted(cdf, u).clamp_(max=domain - 1)
    # SplitMix64-style mixing in int64 arithmetic (wrapping multiplies).
    x = r * 0x100000001B3 + salt
    x = x ^ (x >> 30) & 0x3FFFFFFFF
    x = x * -4658895280553007687  # 0xBF58476D1CE4E5B9 as int64
    x = x ^ ((x >> 27) & 0x1FFFFFFFFF)
    x = x * -7723592293110705685  # 0x94D049BB133111EB as int64
    return x ^ ((x >> 31) & 0x1FFFFFFFF)


def plain_record(torch, keys, L, stream=None):
    """(sizing record, groups) of the plain operator (AUTO sizing) on a device key column."""
    fac = omg.HashAggregationOperatorFactory([0], [L], [[]], [[]], [[L]], [omg.OMNI_AGGREGATION_TYPE_COUNT_ALL])
    op = fac.create_operator()
    if stream is not None:
        op.set_stream(stream)
    op.set_device_output(True)
    op.add_input(omg.wrap_device_batch([L], keys.numel(), [keys.data_ptr()]))
    outs, _ = op.get_outputs(1 << 16)
    omg.free_batches(outs)
    rec, groups = sz.record_from_operator(op)
    op.delete()
    fac.close()
    return rec, groups


def collect(torch, count: int, seed: int, n_min=1 << 20, n_max=1 << 28, d_max=1 << 27, log=print):
    """Sizing records of `count` workloads: N log-uniform in [n_min, n_max], the key domain a
    log-uniform fraction 2^-12 .. 2 of N (at least 10, at most d_max), Zipf(s in [0.7, 1.4]) by
    rank for 70% of them, uniform otherwise."""
    dev = torch.device("cuda", torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    rng = np.random.default_rng(seed)
    L = omg.LongType()
    records = []
    t0 = time.time()
    for i in range(count):
        n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        domain = int(min(d_max, max(10, n * 2.0 ** rng.uniform(-12, 1))))
        kind = "zipf" if rng.random() < 0.7 else "uniform"
        s = float(rng.uniform(0.7, 1.4))
        keys = gpu_keys(torch, gen, n, domain, kind, s, int(rng.integers(0, 2**31)), dev)
        torch.cuda.synchronize()
        rec, groups = plain_record(torch, keys, L)
        records.append((rec, groups, dict(n=n, domain=domain, kind=kind, s=s)))
        del keys
        if log and (i + 1) % 25 == 0:
            log(f"  {i + 1}/{count} records ({time.time() - t0:.1f} s)")
    return records


def make_tasks(torch, n_tasks: int, seed: int, dev, rows_min=1000, rows_max=1_000_000, d_max=1_000_000):
    """Batched-task workload on the GPU: per task, rows log-uniform in [rows_min, rows_max] and a
    key domain log-uniform in [10, min(rows, d_max)], uniform keys; an int64 value column.
    Returns (keys, values, per-task (offset, rows)) with all tasks in two device tensors."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    rows = np.exp(rng.uniform(math.log(rows_min), math.log(rows_max), n_tasks)).astype(np.int64)
    doms = np.exp(rng.uniform(math.log(10), np.log(np.minimum(rows, d_max)))).astype(np.int64)
    doms = np.maximum(doms, 2)
    offs = np.concatenate([[0], np.cumsum(rows)])
    keys = torch.empty(int(offs[-1]), dtype=torch.int64, device=dev)
    for t in range(n_tasks):
        keys[offs[t]:offs[t + 1]] = gpu_keys(torch, gen, int(rows[t]), int(doms[t]), "uniform", 0.0, t * 7919 + seed,
                                             dev)
    vals = torch.randint(-10**6, 10**6, (int(offs[-1]),), generator=gen, device=dev, dtype=torch.int64)
    return keys, vals, [(int(offs[t]), int(rows[t])) for t in range(n_tasks)]


def collect_tasks(torch, n_tasks: int, seed: int, **kw):
    """Per-task sizing records logged by a plain batched run (SUM and COUNT of an int64 value by
    an int64 key, the batched-task plan)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    keys, vals, spans = make_tasks(torch, n_tasks, seed, dev, **kw)
    torch.cuda.synchronize()
    L = omg.LongType()
    fac = omg.HashAggregationOperatorFactory([0], [L], [[1], [1]], [[L], [L]], [[L], [L]],
                                             [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN])
    batches = [omg.wrap_device_batch([L, L], n, [keys.data_ptr() + 8 * o, vals.data_ptr() + 8 * o]) for o, n in spans]
    b = omg.AggBatch(fac, batches, flags=omg.BATCH_DEVICE_OUTPUT)
    b.run()
    omg.free_batches([x for _, x in b.outputs()])
    logs = b.sizing_logs()
    b.close()
    omg.free_batches(batches)
    fac.close()
    return [(lg[:22], lg[19], {}) for lg in logs]


def train(records, epochs=4000, lr=3e-3, seed=1):
    X, T = sz.dataset([(r, g) for r, g, _ in records])
    m = sz.SizingModel(seed=seed)
    loss = m.train(X, T, epochs=epochs, lr=lr)
    return m, loss


def evaluate(m, records):
    """Mean |log2(estimate / groups)| of the model and of the plain estimate."""
    X, _ = sz.dataset([(r, g) for r, g, _ in records])
    y = m.predict(X)
    learned = [abs(math.log2(sz.estimate(r, v) / g)) for (r, g, _), v in zip(records, y)]
    plain = [abs(math.log2(max(r[20], 1) / g)) for r, g, _ in records]
    return float(np.mean(learned)), float(np.mean(plain))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--train", type=int, default=320)
    ap.add_argument("--test", type=int, default=60)
    ap.add_argument("--epochs", type=int, default=4000)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--n-max-log2", type=int, default=28, help="largest workload, log2 rows")
    ap.add_argument("--tasks", action="store_true",
                    help="train on the per-task records of batched runs (the batched-task sizer)")
    a = ap.parse_args(argv)
    import torch

    torch.cuda.init()
    if a.tasks:
        print(f"collecting per-task sizing records from plain batched runs ({a.train}0 + {a.test}0 tasks)")
        tr = collect_tasks(torch, 10 * a.train, a.seed)
        te = collect_tasks(torch, 10 * a.test, a.seed + 1)
    else:
        print(f"collecting {a.train} training and {a.test} held-out sizing records from the plain operator")
        tr = collect(torch, a.train, a.seed, n_max=1 << a.n_max_log2)
        te = collect(torch, a.test, a.seed + 1, n_max=1 << a.n_max_log2)
    m, loss = train(tr, epochs=a.epochs)
    lt, pt = evaluate(m, te)
    print(f"train loss {loss:.5f}; held-out mean |log2 error|: learned {lt:.3f}, plain {pt:.3f}")
    m.save(a.out)
    print(f"saved {a.out}")


if __name__ == "__main__":
    main()
