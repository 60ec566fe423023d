"""Benchmark of the GB300 hash join probe (headline) and hash aggregation (secondary).

Headline workload (one GPU): inner hash join, build 2^20 unique int64 keys (a seeded permutation
of 0..2^20-1) with two uniform int32 payloads; probe 2^26 int64 keys, 1% NULL, 80% drawn from
the build keys, the rest from [2^20, 2^21) (never matching); output (probe key, p1, p2).
A step is one LookupJoin pass over the 2^26 probe rows against the resident build table.

  value  rows/s with inputs resident in HBM (device VectorBatch views over torch memory),
         output left in HBM (device output batches);
  e2e    rows/s through the same C ABI with HOST (pinned) VectorBatches of 4096 rows in and
         host VectorBatches out, the operator pipelined (setNoMoreInput(false) ... noMoreInput()).
Inputs and outputs (0.55 GB + 0.85 GB per step) exceed the 129 MB L2, so no flush is needed.

The "agg" object reports the uniform-key HashAggregation the same way: 2^22 rows, int64 key
over 10,000 distinct values, SUM/COUNT/MIN/MAX(int64), SUM/AVG(double); its 101 MB input fits
in L2, so a 512 MB buffer is rewritten between its timed steps.

Further objects, each a workload of its own with its own timing:
  agg_skewed   2^28 rows, (int32, int64) key Zipf(1.1) over 50M pairs, SUM(decimal64) ->
               decimal128, COUNT(*), AVG(double), 2% NULLs: the table sized by the plain sketch
               estimate vs by the learned sizing model vs by the exact group count;
  agg_batched  10,000 independent aggregations (1e3-1e6 rows each, SUM and COUNT): one operator
               per task (a sample) vs one batched, graph-replayed launch sized plainly or by the
               learned task sizer;
  join_skewed  build 2^26 (16-byte payload), probe 2^30 Zipf(s), s in {0.9, 1.1, 1.3}: the direct
               probe vs hash partitioning vs learned range partitioning (4096 partitions), every
               output checked against the direct probe's by a row-multiset fingerprint;
  join_kinds   the headline data through left outer, left semi, left anti, existence and full
               outer joins (with the outer-join operator), and an inner join on a two-column key;
  agg_two_stage  the uniform aggregation as 4 partial + 1 final operator, and AlignSchema.
Inputs of these legs are larger than L2.

`--impl reference` times the reference's CPU algorithm (the oracle restatement; the reference
itself does not build) on all host cores for the headline workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# omg_debug_last_probe_kernel codes
PROBE_KERNEL_NAMES = {1: "ProbeKindKernel", 2: "ProbeKernel", 3: "ProbeFastKernel", 4: "ProbeBitsKernel",
                      5: "ProbeGroupKernel", 6: "ProbeBulkKernel"}
N_BUILD = 1 << 20
N_PROBE = 1 << 26
AGG_ROWS = 1 << 22
AGG_GROUPS = 10_000
BATCH = 4096
METRIC = "rows/s and HBM-roofline % for hash agg & join probe; learned vs plain, bit-exact"
JOIN_WORKLOAD = ("inner hash join probe: build 2^20 unique int64 keys + 2 int32 payloads, probe 2^26 int64 "
                 "keys (1% null, 80% match) in 4096-row batches, output (probe key, p1, p2)")


_T0 = time.perf_counter()


def log(msg):
    """Progress of the run on stderr (elapsed seconds), so that a slow leg can be found."""
    print(f"[bench {time.perf_counter() - _T0:8.1f} s] {msg}", file=sys.stderr, flush=True)


def measured_peak_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def profiled_traffic(name):
    """DRAM bytes per unit from a committed ncu summary (a `traffic_bytes_per_unit:` line)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        s = line.strip().lstrip("-* ")
        if s.startswith("traffic_bytes_per_unit:"):
            try:
                return float(s.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={','.join(self.FIELDS)}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(self.NAMES, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------ data (host)
def join_data_numpy(seed, n_probe=N_PROBE):
    rng = np.random.default_rng(seed)
    bkey = rng.permutation(N_BUILD).astype(np.int64)
    p1 = rng.integers(-2**31, 2**31, N_BUILD, dtype=np.int64).astype(np.int32)
    p2 = rng.integers(-2**31, 2**31, N_BUILD, dtype=np.int64).astype(np.int32)
    match = rng.random(n_probe) < 0.8
    pkey = np.where(match, bkey[rng.integers(0, N_BUILD, n_probe)],
                    rng.integers(N_BUILD, 2 * N_BUILD, n_probe)).astype(np.int64)
    pnull = rng.random(n_probe) < 0.01
    return bkey, p1, p2, pkey, pnull


def agg_data_numpy(seed):
    rng = np.random.default_rng(seed)
    uniq = rng.integers(-2**62, 2**62, AGG_GROUPS, dtype=np.int64)
    key = uniq[rng.integers(0, AGG_GROUPS, AGG_ROWS)]
    v1 = rng.integers(-10**6, 10**6 + 1, AGG_ROWS, dtype=np.int64)
    v2 = rng.random(AGG_ROWS)
    return key, v1, v2


# ------------------------------------------------------------------------------ CPU (oracle) timing
def cpu_join_rows_per_s(data, threads, reps=1):
    import oracle

    L = oracle.lib()
    bkey, p1, p2, pkey, pnull = data
    pn = pnull.astype(np.uint8)
    pays = (C.c_void_p * 2)(p1.ctypes.data, p2.ctypes.data)
    times = []
    secs = (C.c_double * 2)()
    for _ in range(reps):
        n = L.orc_join_probe_bench(N_BUILD, bkey.ctypes.data, None, 2, pays, len(pkey), pkey.ctypes.data,
                                   pn.ctypes.data, threads, secs)
        times.append(secs[1])  # the probe; the build is timed separately, as on the GPU
        assert n > 0
    return len(pkey) / statistics.median(times)


def cpu_agg_rows_per_s(data, threads, reps=1):
    import oracle

    L = oracle.lib()
    key, v1, v2 = data
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        g = L.orc_agg_bench(len(key), key.ctypes.data, v1.ctypes.data, v2.ctypes.data, threads)
        times.append(time.perf_counter() - t0)
        assert g == AGG_GROUPS
    return len(key) / statistics.median(times)


# ------------------------------------------------------------------------------ parity at full size
# The oracle is the checker here: every check runs outside the timed regions, on the same
# inputs as the timed steps, and its verdict goes into the bench line as "oracle_match".
DOUBLE_TOL = 1e-12


def host_threads():
    return os.cpu_count() or 1


def mem_available_bytes():
    """MemAvailable of this host (bytes), or None when unknown."""
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def host_columns(omg, batches):
    """Concatenated [(values, NULL mask)] of host output batches (frees them)."""
    parts = []
    for b in batches:
        parts.append(omg.batch_to_numpy(b))
        omg.free_batch(b)
    if not parts:
        return None
    return [(np.concatenate([p[c][0] for p in parts]), np.concatenate([p[c][1] for p in parts]))
            for c in range(len(parts[0]))]


def _key_order(keys, masks):
    """Row order sorting by the key columns (NULL first per column)."""
    parts = []
    for v, m in zip(keys, masks):
        m = np.asarray(m, dtype=bool)
        parts.append(np.where(m, 0, np.asarray(v).astype(np.int64)))
        parts.append(~m)
    return np.lexsort(parts[::-1])


def compare_agg_full(gpu_cols, ora, nkeys, double_aggs):
    """Compare GPU output columns [(values, mask)] with oracle.hashagg_mt's result group for
    group: keys, integer / decimal / COUNT / MIN / MAX values and NULLs bit-exact; the double
    SUM / AVG aggregates in `double_aggs` ({output index: (oracle exact index, divisor index or
    None)}) within 1e-12 * max(|exact|, sum|x|) (divided by the non-NULL count for AVG) of the
    double-double sum.  Returns a summary dict with "oracle_match"."""
    okeys, oknulls, ovals, onulls, oexact, oabs = ora
    ng = len(okeys[0])
    res = {"groups": ng}
    if gpu_cols is None or len(gpu_cols[0][0]) != ng:
        res.update(oracle_match=False, why=f"group count {0 if gpu_cols is None else len(gpu_cols[0][0])} != {ng}")
        return res
    go = _key_order([c[0] for c in gpu_cols[:nkeys]], [c[1] for c in gpu_cols[:nkeys]])
    oo = _key_order(okeys, oknulls)
    for k in range(nkeys):
        gv, gm = gpu_cols[k][0][go], gpu_cols[k][1][go]
        ov, om = okeys[k][oo], oknulls[k][oo]
        if not np.array_equal(gm, om) or not np.array_equal(np.where(gm, 0, gv), np.where(om, 0, ov)):
            res.update(oracle_match=False, why=f"key column {k} differs")
            return res
    worst = 0.0
    naive = 0.0
    for j in range(len(gpu_cols) - nkeys):
        gv, gm = gpu_cols[nkeys + j][0][go], gpu_cols[nkeys + j][1][go]
        ov, om = ovals[j][oo], onulls[j][oo]
        if not np.array_equal(gm, om):
            res.update(oracle_match=False, why=f"NULLs of aggregate {j} differ")
            return res
        live = ~gm
        if j in double_aggs:
            ei, di = double_aggs[j]
            ex, ab = oexact[ei][oo][live], oabs[ei][oo][live]
            div = np.ones(int(live.sum())) if di is None else ovals[di][oo][live].astype(np.float64)
            target = ex / div
            tol = DOUBLE_TOL * np.maximum(np.abs(ex), ab) / div
            tol = np.where(tol > 0, tol, np.finfo(np.float64).tiny)
            err = np.abs(gv[live].astype(np.float64) - target)
            worst = max(worst, float((err / tol).max()) if len(err) else 0.0)
            scale = np.maximum(np.abs(ex), ab) / div
            scale = np.where(scale > 0, scale, 1.0)
            naive = max(naive, float((np.abs(ov[live].astype(np.float64) - target) / scale).max()) if len(err) else 0.0)
        else:
            a = np.asarray(gv[live])
            b = np.asarray(ov[live])
            if a.ndim == 2 or b.ndim == 2:
                same = np.array_equal(a.view(np.uint64).reshape(-1, 2), b.view(np.uint64).reshape(-1, 2))
            else:
                same = np.array_equal(a.astype(np.int64), b.astype(np.int64))
            if not same:
                if a.ndim == 2 or b.ndim == 2:
                    bad = np.nonzero((a.view(np.uint64).reshape(-1, 2) != b.view(np.uint64).reshape(-1, 2)).any(1))[0]
                else:
                    bad = np.nonzero(a.astype(np.int64) != b.astype(np.int64))[0]
                rows = np.nonzero(live)[0][bad[:3]]
                sample = [{"keys": [str(gpu_cols[k][0][go][r]) for k in range(nkeys)],
                           "gpu": str(gpu_cols[nkeys + j][0][go][r].tolist()), "oracle": str(ovals[j][oo][r].tolist())}
                          for r in rows]
                res.update(oracle_match=False, why=f"aggregate {j} differs in {len(bad)} groups", sample=sample)
                return res
    res.update(oracle_match=worst <= 1.0, double_err_over_tol=round(worst, 6))
    if double_aggs:
        res["reference_fold_max_rel_err"] = float(f"{naive:.3g}")
    return res


def base_line(args, value, ms):
    return {"metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded)"}


def run_reference(args, rank):
    if rank != 0:
        return
    import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    data = join_data_numpy(1)
    for _ in range(args.warmup):
        cpu_join_rows_per_s(data, threads)
    vals, t0 = [], time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_join_rows_per_s(data, threads))
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    line = base_line(args, value, 1e3 * wall / max(args.steps, 1))
    line.update({"impl": "reference",
                 "config": {"workload": JOIN_WORKLOAD,
                            "implementation": "CPU restatement of the reference's build/probe loops (oracle/oracle.c); "
                                              "the reference needs jemalloc, securec, LLVM and its CMake build"},
                 "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                                  "sample": f"full workload (2^26 probe rows) per step, {threads} threads"},
                 "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    print(json.dumps(line), flush=True)


def replica_sync(dist, device):
    """barrier() and max_over_ranks(x) for N independent replicas (one process per GPU, no
    data-path collective): the timed region is bracketed by barriers and each rank's elapsed
    time is reduced with MAX, so a whole-job rate is world * units per rank / that maximum.
    `dist` is torch.distributed (None for one process); `device` holds the reduction tensor (the
    rank's GPU, or the CPU under gloo)."""
    import torch

    def barrier():
        if dist is not None:
            dist.barrier()
        if device.type == "cuda":
            torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def whole_job_rate(world, units_per_rank, seconds):
    """Units all ranks processed per second of the slowest rank."""
    return world * units_per_rank / seconds


# ------------------------------------------------------------------------------ GPU arm
def run_gpu(args, rank, world):
    import torch

    import omnioperator_gb300 as omg
    from omnioperator_gb300 import build as omg_build

    omg_build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    barrier, max_over_ranks = replica_sync(dist, dev)

    L, I, D = omg.LongType(), omg.IntType(), omg.DoubleType()
    stream = torch.cuda.current_stream()
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    if args.only == "agg":
        agg = run_agg(args, omg, torch, dev, stream, barrier, max_over_ranks, world)
        return dict(value=agg["value"], ms=agg["ms_per_step"], build_ms=0.0, launches=agg["gpu_launches"],
                    roofline=agg["roofline"], clocks=None, e2e=None, agg=agg, rows=AGG_GROUPS, skew=None,
                    batched=None, join5=None)
    if args.only == "join5":
        j5 = run_join_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank)
        d = j5["s=1.1"]["learned_choice"]
        return dict(value=d["value"], ms=d["ms_per_step"], build_ms=0.0, launches=0, roofline=None, clocks=None,
                    e2e=None, agg=None, rows=d["output_rows"], skew=None, batched=None, join5=j5)
    if args.only == "batched":
        bt = run_agg_batched(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank)
        arm = bt.get("batched_learned", bt["batched_plain"])
        return dict(value=arm["value"], ms=arm["ms_per_step"], build_ms=0.0, launches=0, roofline=None, clocks=None,
                    e2e=None, agg=None, rows=arm["groups"], skew=None, batched=bt, join5=None)
    if args.only == "skew":
        sk = run_agg_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank)
        return dict(value=sk["learned"]["value"], ms=sk["learned"]["ms_per_step"], build_ms=0.0, launches=0,
                    roofline=None, clocks=None, e2e=None, agg=None, rows=sk["learned"]["groups"], skew=sk,
                    batched=None, join5=None)

    # ---- device-resident join inputs (torch tensors seen as OmniVec device vectors)
    bkey = torch.randperm(N_BUILD, generator=g, device=dev).to(torch.int64)
    p1 = torch.randint(-2**31, 2**31 - 1, (N_BUILD,), generator=g, device=dev, dtype=torch.int32)
    p2 = torch.randint(-2**31, 2**31 - 1, (N_BUILD,), generator=g, device=dev, dtype=torch.int32)
    match = torch.rand(N_PROBE, generator=g, device=dev) < 0.8
    pick = torch.randint(0, N_BUILD, (N_PROBE,), generator=g, device=dev)
    miss = torch.randint(N_BUILD, 2 * N_BUILD, (N_PROBE,), generator=g, device=dev)
    pkey = torch.where(match, bkey[pick], miss).contiguous()
    pnull = torch.rand(N_PROBE, generator=g, device=dev) < 0.01
    weights = torch.tensor([1, 2, 4, 8, 16, 32, 64, 128], device=dev, dtype=torch.int32)
    pbits = (pnull.view(-1, 8).to(torch.int32) * weights).sum(1).to(torch.uint8)
    pbits = torch.cat([pbits, torch.zeros(16, dtype=torch.uint8, device=dev)])
    expected_rows = int((match & ~pnull).sum().item())
    del match, pick, miss

    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I, I], [0])
    bop = bf.create_operator()
    bop.set_stream(stream.cuda_stream)
    bop.add_input(omg.wrap_device_batch([L, I, I], N_BUILD, [bkey.data_ptr(), p1.data_ptr(), p2.data_ptr()]))
    torch.cuda.synchronize()
    tb0 = time.perf_counter()
    bop.get_output()
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - tb0) * 1e3
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf)
    pop = pf.create_operator()
    pop.set_stream(stream.cuda_stream)
    pop.set_device_output(True)
    omg.lib().omg_debug_set_bulk_probe(args.bulk_probe)

    def probe_step():
        pop.add_input(omg.wrap_device_batch([L], N_PROBE, [pkey.data_ptr()], [pbits.data_ptr()]))
        outs, rows = pop.get_outputs(1 << 16)  # GetOutput until drained, one C call
        omg.free_batches(outs)
        return rows

    for _ in range(args.warmup):
        rows = probe_step()
        assert rows == expected_rows, (rows, expected_rows)
    # Parity at full size (outside the timed steps): the row-multiset fingerprint of one probe
    # pass against the oracle's join of the same build and probe rows.
    pop.add_input(omg.wrap_device_batch([L], N_PROBE, [pkey.data_ptr()], [pbits.data_ptr()]))
    outs, _ = pop.get_outputs(1 << 16)
    gpu_fp = omg.batches_fingerprint(outs)
    omg.free_batches(outs)
    join_check = check_join_fingerprint(gpu_fp, bkey.cpu().numpy(), [p1.cpu().numpy(), p2.cpu().numpy()],
                                        pkey.cpu().numpy(), pnull.cpu().numpy())
    c0 = pop.counters()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            rows = probe_step()
        ev1.record(stream)
        barrier()
    assert rows == expected_rows
    c1 = pop.counters()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    value = whole_job_rate(world, N_PROBE * args.steps, ms / 1e3)
    kernel_s = (c1["kernel_ns"] - c0["kernel_ns"]) / max(c1["kernel_launches"] - c0["kernel_launches"], 1) / 1e9
    launches = c1["launches"] - c0["launches"]
    # Algorithmic bytes of one probe launch: 8 B key + 1/8 B validity per probe row, 16 B per output row.
    alg_bytes = N_PROBE * 8 + N_PROBE / 8 + expected_rows * 16
    peak, peak_kind = measured_peak_gbs()
    achieved = alg_bytes / kernel_s / 1e9
    traffic_per_row = profiled_traffic("probe_kernel_join2e26.md")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": None if traffic_per_row is None else traffic_per_row * N_PROBE,
                "kernel": PROBE_KERNEL_NAMES.get(omg.lib().omg_debug_last_probe_kernel(), "?"),
                "kernel_ms": round(kernel_s * 1e3, 4),
                "algorithmic_bytes": int(alg_bytes)}

    omg.lib().omg_debug_set_bulk_probe(0)
    log(f"headline probe timed ({ms / args.steps:.3f} ms per step), oracle match {join_check['oracle_match']}")
    e2e = None if args.skip_e2e else run_e2e(args, omg, bf, torch, barrier, max_over_ranks, world, rank)
    log("e2e done")
    kinds = None if args.skip_ext else run_join_kinds(args, omg, torch, stream, barrier, max_over_ranks, world, bkey,
                                                       p1, p2, pkey, pbits, pnull)
    log("join kinds done")
    agg = None if args.skip_agg else run_agg(args, omg, torch, dev, stream, barrier, max_over_ranks, world)
    log("uniform aggregation done")
    two_stage = None if args.skip_ext else run_agg_two_stage(args, omg, torch, dev, stream, barrier, max_over_ranks,
                                                              world)
    log("two-stage aggregation done")
    features = None if args.skip_ext else run_features(args, omg, torch, dev, stream, barrier, max_over_ranks, world,
                                                        bf, pkey, pbits)
    pop.delete()
    bop.delete()
    pf.close()
    bf.close()
    del bkey, p1, p2, pkey, pnull, pbits
    log("features done")
    skew = None if args.skip_skew else run_agg_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks,
                                                       world, rank)
    log("skewed aggregation done")
    batched = None if args.skip_batched else run_agg_batched(args, omg, torch, dev, stream, barrier, max_over_ranks,
                                                              world, rank)
    log("batched aggregation done")
    join5 = None if args.skip_join5 else run_join_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks,
                                                          world, rank)
    return dict(value=value, ms=ms / args.steps, build_ms=build_ms, launches=launches, roofline=roofline,
                clocks=clk.summary(), e2e=e2e, agg=agg, rows=expected_rows, skew=skew, batched=batched, join5=join5,
                kinds=kinds, two_stage=two_stage, features=features, join_check=join_check)


def check_join_fingerprint(gpu_fp, bkey, pays, pkey, pnull, table=None):
    """Inner-join output of the GPU (its fingerprint) against the oracle's join of the same
    rows: equal row counts and equal 128-bit row-multiset fingerprints."""
    import oracle

    oracle.build()
    t0 = time.perf_counter()
    jt = table if table is not None else oracle.JoinTable(bkey)
    fp, probe_s = jt.fingerprint(pays, pkey, pnull, threads=host_threads())
    if table is None:
        jt.close()
    return {"oracle_match": tuple(gpu_fp) == tuple(fp), "rows": int(fp[0]), "gpu_rows": int(gpu_fp[0]),
            "fingerprint": f"{fp[1]:016x}{fp[2]:016x}", "check_s": round(time.perf_counter() - t0, 2),
            "oracle_probe_s": round(probe_s, 3)}


def run_join_kinds(args, omg, torch, stream, barrier, max_over_ranks, world, bkey, p1, p2, pkey, pbits, pnull):
    """The headline build and probe data through the other join kinds: outer (probe side),
    semi, anti, existence, full (probe plus the outer-join operator), and an inner join on a
    two-column key (the probe key split into two int32 columns).  Inputs resident in HBM,
    outputs left in HBM; the probe kernel's roofline counts 8 B key + 1/8 B validity per probe
    row and the output bytes."""
    L, I = omg.LongType(), omg.IntType()
    matched = int(((pkey < N_BUILD) & ~pnull).sum().item())
    hits = torch.zeros(N_BUILD, dtype=torch.bool, device=pkey.device)
    hits[pkey[(pkey < N_BUILD) & ~pnull]] = True
    unmatched_build = N_BUILD - int(hits.sum().item())
    del hits
    bhi, blo = (bkey >> 10).to(torch.int32), (bkey & 1023).to(torch.int32)
    phi, plo = (pkey >> 10).to(torch.int32), (pkey & 1023).to(torch.int32)
    cases = [
        # name, join type, probe output cols, build output cols, output row bytes, probe-operator rows
        ("left_outer", omg.OMNI_JOIN_TYPE_LEFT, [0], [1, 2], 16, N_PROBE),
        ("left_semi", omg.OMNI_JOIN_TYPE_LEFT_SEMI, [0], [], 8, matched),
        ("left_anti", omg.OMNI_JOIN_TYPE_LEFT_ANTI, [0], [], 8, N_PROBE - matched),
        ("existence", omg.OMNI_JOIN_TYPE_EXISTENCE, [0], [], 9, N_PROBE),
        ("full_outer", omg.OMNI_JOIN_TYPE_FULL, [0], [1, 2], 16, N_PROBE),
        ("inner_two_column_key", omg.OMNI_JOIN_TYPE_INNER, [0, 1], [2, 3], 16, matched),
    ]
    peak, peak_kind = measured_peak_gbs()
    out = {"workload": "the headline build (2^20) and probe (2^26) data, per join kind; inputs and outputs in HBM"}
    for name, jt, pout, bout, row_bytes, rows in cases:
        two = name == "inner_two_column_key"
        btypes = [I, I, I, I] if two else [L, I, I]
        bcols = [bhi, blo, p1, p2] if two else [bkey, p1, p2]
        bf = omg.HashBuilderOperatorFactory(jt, btypes, [0, 1] if two else [0])
        bop = bf.create_operator()
        bop.set_stream(stream.cuda_stream)
        bop.add_input(omg.wrap_device_batch(btypes, N_BUILD, [c.data_ptr() for c in bcols]))
        bop.get_output()
        ptypes = [I, I] if two else [L]
        pcols = [phi, plo] if two else [pkey]
        pnulls = [pbits.data_ptr(), None] if two else [pbits.data_ptr()]
        bo_types = [btypes[c] for c in bout]
        pf = omg.LookupJoinOperatorFactory(ptypes, pout, [0, 1] if two else [0], bout, bo_types, bf)
        of = (omg.LookupOuterJoinOperatorFactory(ptypes, pout, bout, bo_types, bf)
              if jt == omg.OMNI_JOIN_TYPE_FULL else None)
        pop = pf.create_operator()
        pop.set_stream(stream.cuda_stream)
        pop.set_device_output(True)

        def step():
            pop.add_input(omg.wrap_device_batch(ptypes, N_PROBE, [c.data_ptr() for c in pcols], pnulls))
            outs, n = pop.get_outputs(1 << 16)
            omg.free_batches(outs)
            n_outer = 0
            if of is not None:
                oop = of.create_operator()
                oop.set_stream(stream.cuda_stream)
                oop.set_device_output(True)
                for b in oop.drain():
                    n_outer += omg.batch_row_count(b)
                    omg.free_batch(b)
                oop.delete()
            return n, n_outer

        for _ in range(args.warmup):
            n, n_outer = step()
            assert n == rows and n_outer == (unmatched_build if of is not None else 0), (name, n, n_outer)
        c0 = pop.counters()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            n, n_outer = step()
        e1.record(stream)
        barrier()
        c1 = pop.counters()
        ms = max_over_ranks(e0.elapsed_time(e1)) / args.steps
        kernel_s = (c1["kernel_ns"] - c0["kernel_ns"]) / max(c1["kernel_launches"] - c0["kernel_launches"], 1) / 1e9
        alg = (N_PROBE * (8 if not two else 8) + N_PROBE / 8 + rows * row_bytes)
        achieved = alg / kernel_s / 1e9
        out[name] = {"value": world * N_PROBE / (ms / 1e3), "unit": "probe rows/s", "ms_per_step": round(ms, 4),
                     "output_rows": n, "outer_rows": n_outer,
                     "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                                  "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                                  "kernel": PROBE_KERNEL_NAMES.get(omg.lib().omg_debug_last_probe_kernel(), "?"),
                                  "kernel_ms": round(kernel_s * 1e3, 4),
                                  "algorithmic_bytes": int(alg)}}
        pop.delete()
        bop.delete()
        if of is not None:
            of.close()
        pf.close()
        bf.close()
    return out


def run_features(args, omg, torch, dev, stream, barrier, max_over_ranks, world, bf, pkey_t, pnull_bits):
    """Throughput of the operator features beyond the two headline plans, each timed with CUDA
    events around whole operator calls (host work included), inputs in HBM:
    * agg_varchar: 2^22 rows grouped by a VARCHAR key over 10,000 distinct strings of 8-24 bytes,
      SUM and COUNT of an int64 column (string dictionary, aggregation on ids, strings restored);
    * join_filter: the headline probe (2^26 rows) with the filter build.p1 >= 0 (about half the
      matches pass), evaluated in the bitmap probe on each row's one candidate, with the kernel's
      roofline (8 B key + 1/8 B validity per probe row and 16 B per output row);
    * agg_spill: the uniform aggregation (2^22 rows) with a 256 KiB device budget, so its rows are
      partitioned into pinned host memory and aggregated one partition at a time, next to the
      unspilled run."""
    L, I, D, V = omg.LongType(), omg.IntType(), omg.DoubleType(), omg.VarcharType(24)
    SUM, CNT, MIN, MAX, AVG = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                               omg.OMNI_AGGREGATION_TYPE_MIN, omg.OMNI_AGGREGATION_TYPE_MAX,
                               omg.OMNI_AGGREGATION_TYPE_AVG)
    out = {"workload": "operator features, inputs in HBM, whole operator calls timed: VARCHAR group-by keys "
                       "(2^22 rows, 10,000 strings), a join filter on the headline probe (2^26 rows), "
                       "aggregation spill (2^22 rows, 256 KiB device budget)"}

    def timed(fn, n_steps, n_warm):
        for _ in range(n_warm):
            fn()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n_steps):
            fn()
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(time.perf_counter() - t0) / n_steps

    # VARCHAR keys
    rng = np.random.default_rng(5)
    words = [bytes(rng.integers(97, 123, l, dtype=np.uint8)) for l in rng.integers(8, 25, 10_000)]
    idx = rng.integers(0, len(words), AGG_ROWS)
    keys = np.array([words[i] for i in idx], dtype=object)
    vals = rng.integers(-10**6, 10**6, AGG_ROWS, dtype=np.int64)
    host = omg.make_batch([V, L], [keys, vals])
    fac = omg.HashAggregationOperatorFactory([0], [V], [[1], [1]], [[L], [L]], [[L], [L]], [SUM, CNT])
    n_steps, n_warm = max(1, min(args.steps, 5)), max(1, min(args.warmup, 2))
    dev_batches = [omg.batch_to_device(host) for _ in range(n_steps + n_warm)]
    omg.free_batch(host)
    groups = []

    def agg_varchar():
        op = fac.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        op.add_input(dev_batches.pop())
        outs = op.drain()
        groups.append(sum(omg.batch_row_count(b) for b in outs))
        omg.free_batches(outs)
        op.delete()

    t = timed(agg_varchar, n_steps, n_warm)
    fac.close()
    assert all(g == len(set(idx.tolist())) for g in groups)
    out["agg_varchar"] = {"value": world * AGG_ROWS / t, "unit": "rows/s", "ms_per_step": round(t * 1e3, 3),
                          "groups": groups[-1]}

    # join filter over the headline build and probe
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf,
                                       filter_expr=omg.Binary(omg.EXPR_GTE, omg.Field(2, I), omg.Literal(0, I)))
    rows = []
    kern = []

    def join_filter():
        op = pf.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        op.add_input(omg.wrap_device_batch([L], N_PROBE, [pkey_t.data_ptr()], [pnull_bits.data_ptr()]))
        outs = op.drain()
        rows.append(sum(omg.batch_row_count(b) for b in outs))
        omg.free_batches(outs)
        c = op.counters()
        kern.append(c["kernel_ns"] / max(c["kernel_launches"], 1) / 1e9)
        op.delete()

    t = timed(join_filter, max(1, min(args.steps, 5)), n_warm)
    pf.close()
    kernel_s = float(np.median(kern[n_warm:] or kern))
    alg = N_PROBE * 8 + N_PROBE / 8 + rows[-1] * 16
    peak, peak_kind = measured_peak_gbs()
    out["join_filter"] = {"value": world * N_PROBE / t, "unit": "probe rows/s", "ms_per_step": round(t * 1e3, 3),
                          "output_rows": rows[-1],
                          "roofline": {"bound": "hbm", "achieved": round(alg / kernel_s / 1e9, 1), "peak": peak,
                                       "unit": "GB/s", "frac": round(alg / kernel_s / 1e9 / peak, 4),
                                       "peak_kind": peak_kind,
                                       "kernel": PROBE_KERNEL_NAMES.get(omg.lib().omg_debug_last_probe_kernel(), "?"),
                                       "kernel_ms": round(kernel_s * 1e3, 4), "algorithmic_bytes": int(alg)}}

    # spill
    key, v1, v2 = agg_data_numpy(2)
    tk, t1, t2 = (torch.from_numpy(x).to(dev) for x in (key, v1, v2))
    afac = omg.HashAggregationOperatorFactory(
        [0], [L], [[1], [1], [1], [1], [2], [2]], [[L], [L], [L], [L], [D], [D]], [[L], [L], [L], [L], [D], [D]],
        [SUM, CNT, MIN, MAX, SUM, AVG])
    spilled = []

    def agg(budget):
        def run():
            op = afac.create_operator()
            op.set_stream(stream.cuda_stream)
            op.set_device_output(True)
            if budget:
                op.set_spill(True, budget)
            op.add_input(omg.wrap_device_batch([L, L, D], AGG_ROWS, [tk.data_ptr(), t1.data_ptr(), t2.data_ptr()]))
            outs = op.drain()
            assert sum(omg.batch_row_count(b) for b in outs) == AGG_GROUPS
            omg.free_batches(outs)
            spilled.append(op.spilled_bytes())
            op.delete()
        return run

    t_plain = timed(agg(0), n_steps, n_warm)
    t_spill = timed(agg(256 << 10), n_steps, n_warm)
    afac.close()
    out["agg_spill"] = {"value": world * AGG_ROWS / t_spill, "unit": "rows/s", "ms_per_step": round(t_spill * 1e3, 3),
                        "unspilled_ms_per_step": round(t_plain * 1e3, 3), "spilled_bytes": spilled[-1],
                        "device_budget_bytes": 256 << 10}
    return out


def run_agg_two_stage(args, omg, torch, dev, stream, barrier, max_over_ranks, world):
    """The uniform aggregation's data split over 4 partial operators, merged by one final
    operator; and AlignSchema (adaptive partial aggregation) over all 2^22 rows.  Inputs in HBM,
    outputs in HBM, L2 flushed between steps."""
    L, D = omg.LongType(), omg.DoubleType()
    SUM, CNT, MIN, MAX, AVG = (omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN,
                               omg.OMNI_AGGREGATION_TYPE_MIN, omg.OMNI_AGGREGATION_TYPE_MAX,
                               omg.OMNI_AGGREGATION_TYPE_AVG)
    key, v1, v2 = agg_data_numpy(2)
    tk, t1, t2 = (torch.from_numpy(x).to(dev) for x in (key, v1, v2))
    flush = torch.empty(1 << 27, dtype=torch.int32, device=dev)
    funcs = [SUM, CNT, MIN, MAX, SUM, AVG]
    part = omg.HashAggregationOperatorFactory([0], [L], [[1], [1], [1], [1], [2], [2]], [[L]] * 4 + [[D], [D]],
                                              [[L], [L], [L], [L], [D], [D, L]], funcs,
                                              output_partials=[True] * 6)
    fin = omg.HashAggregationOperatorFactory([0], [L], [[1], [2], [3], [4], [5], [6, 7]],
                                             [[L]] * 4 + [[D], [D, L]], [[L]] * 4 + [[D], [D]], funcs,
                                             input_raws=[False] * 6)
    quarter = AGG_ROWS // 4

    def run(fac, batches):
        op = fac.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        for b in batches:
            op.add_input(b)
        outs = op.drain()
        op.delete()
        return outs

    def step():
        partials = []
        for q in range(4):
            o = q * quarter
            partials += run(part, [omg.wrap_device_batch([L, L, D], quarter, [tk.data_ptr() + 8 * o,
                                                                            t1.data_ptr() + 8 * o,
                                                                            t2.data_ptr() + 8 * o])])
        e_mid = torch.cuda.Event(enable_timing=True)
        e_mid.record(stream)
        final = run(fin, partials)
        groups = sum(omg.batch_row_count(b) for b in final)
        omg.free_batches(final)
        return groups, e_mid

    def align_step():
        op = part.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        b = op.align_schema(omg.wrap_device_batch([L, L, D], AGG_ROWS, [tk.data_ptr(), t1.data_ptr(), t2.data_ptr()]))
        n = omg.batch_row_count(b)
        omg.free_batch(b)
        op.delete()
        return n

    for _ in range(args.warmup):
        flush.fill_(1)
        assert step()[0] == AGG_GROUPS
        assert align_step() == AGG_ROWS
    tot = partial_ms = align_ms = 0.0
    for _ in range(args.steps):
        flush.fill_(1)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        groups, e_mid = step()
        e1.record(stream)
        barrier()
        tot += e0.elapsed_time(e1)
        partial_ms += e0.elapsed_time(e_mid)
        assert groups == AGG_GROUPS
        flush.fill_(1)
        barrier()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        assert align_step() == AGG_ROWS
        a1.record(stream)
        barrier()
        align_ms += a0.elapsed_time(a1)
    ms = max_over_ranks(tot) / args.steps
    part.close()
    fin.close()
    peak, kind = measured_peak_gbs()
    align_s = max_over_ranks(align_ms) / args.steps / 1e3
    # AlignSchema moves 24 B in and 72 B out per row (key, SUM, COUNT, MIN, MAX, SUM, AVG sum + count).
    return {"workload": "the uniform aggregation (2^22 rows, 10,000 groups) as 4 partial operators + 1 final "
                        "operator; AlignSchema of all 2^22 rows; L2 flushed between steps",
            "two_stage": {"value": world * AGG_ROWS / (ms / 1e3), "unit": "rows/s", "ms_per_step": round(ms, 4),
                          "partial_ms": round(partial_ms / args.steps, 4),
                          "final_ms": round(ms - partial_ms / args.steps, 4), "partial_rows": 4 * AGG_GROUPS},
            "align_schema": {"value": world * AGG_ROWS / align_s, "unit": "rows/s",
                             "ms_per_step": round(align_s * 1e3, 4),
                             "achieved_gbs": round(AGG_ROWS * 96 / align_s / 1e9, 1), "peak": peak,
                             "frac_of_peak": round(AGG_ROWS * 96 / align_s / 1e9 / peak, 4), "peak_kind": kind}}


def run_e2e(args, omg, bf, torch, barrier, max_over_ranks, world, rank):
    """Same probe through host (pinned) VectorBatches of 4096 rows in, host batches out."""
    L, I = omg.LongType(), omg.IntType()
    bkey, p1, p2, pkey, pnull = join_data_numpy(7 + rank, N_PROBE)
    # The e2e operator probes against a build of this step's host data (same shape, same table kind).
    bf2 = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, I, I], [0])
    bop = bf2.create_operator()
    for s in range(0, N_BUILD, 1 << 16):
        bop.add_input(omg.make_batch([L, I, I], [bkey[s:s + (1 << 16)], p1[s:s + (1 << 16)], p2[s:s + (1 << 16)]]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [I, I], bf2)
    expected = int((~pnull & (pkey < N_BUILD)).sum())

    def make_batches():
        """Host batches of 4096 rows, grouped 1024 to a C array (one AddInput call chain each)."""
        hs = [omg.make_batch([L], [pkey[s:s + BATCH]], [pnull[s:s + BATCH]]) for s in range(0, N_PROBE, BATCH)]
        return [(C.c_void_p * len(hs[i:i + 1024]))(*hs[i:i + 1024]) for i in range(0, len(hs), 1024)]

    fp = [0, 0, 0]

    def step(chunks, fingerprint=False):
        op = pf.create_operator()
        op.set_no_more_input(False)
        rows = 0

        def take(outs):
            if fingerprint and outs:
                f = omg.batches_fingerprint(outs)
                for i in range(3):
                    fp[i] = (fp[i] + f[i]) & ((1 << 64) - 1)
            omg.free_batches(outs)

        for chunk in chunks:
            op.add_inputs(chunk)  # AddInput per batch, in C
            outs, n = op.get_outputs(1 << 16)
            rows += n
            take(outs)
        op.no_more_input()
        outs, n = op.get_outputs(1 << 16)
        rows += n
        take(outs)
        op.delete()
        return rows

    # Parity (outside the timed steps): the host output batches of one pass against the oracle.
    assert step(make_batches(), fingerprint=True) == expected
    check = check_join_fingerprint(fp, bkey, [p1, p2], pkey, pnull)
    for _ in range(max(1, min(args.warmup, 2))):
        assert step(make_batches()) == expected
    total = 0.0
    for _ in range(args.steps):
        batches = make_batches()  # data preparation, outside the timed region
        barrier()
        t0 = time.perf_counter()
        rows = step(batches)
        barrier()
        total += time.perf_counter() - t0
        assert rows == expected
    t = max_over_ranks(total)
    bop.delete()
    pf.close()
    bf2.close()
    h2d = N_PROBE * 8 + N_PROBE // 8
    d2h = expected * 16 + 3 * ((expected + 31) // 32 * 4)
    return {"value": whole_job_rate(world, N_PROBE * args.steps, t), "unit": "rows/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * t / args.steps, "oracle_match": check["oracle_match"],
            "link": link_ceiling(torch, h2d, d2h, t / args.steps)}


def link_ceiling(torch, h2d, d2h, step_s):
    """The CPU-GPU link's measured copy rates (1 GiB pinned <-> HBM, cudaMemcpyAsync, best of 5:
    each direction alone and both at once on two streams) and the e2e step's time against the
    time its host<->device bytes need at those rates (the link roofline of the e2e path)."""
    n = 1 << 30
    host = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(n, dtype=torch.uint8, device="cuda")
    host2 = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    dev2 = torch.empty(n, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def best(fn):
        times = []
        for _ in range(5):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            torch.cuda.synchronize()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        return min(times)

    def both():
        with torch.cuda.stream(s1):
            dev.copy_(host, non_blocking=True)
        with torch.cuda.stream(s2):
            host2.copy_(dev2, non_blocking=True)
        torch.cuda.current_stream().wait_stream(s1)
        torch.cuda.current_stream().wait_stream(s2)

    h2d_s = best(lambda: dev.copy_(host, non_blocking=True))
    d2h_s = best(lambda: host.copy_(dev, non_blocking=True))
    dup_s = best(both)
    h2d_gbs, d2h_gbs, dup_gbs = n / h2d_s / 1e9, n / d2h_s / 1e9, 2 * n / dup_s / 1e9
    # The step's bytes at the link's rates: each direction at its own rate, and the two together at
    # the duplex rate; the slower bound is the floor for this step.
    floor_s = max(h2d / (h2d_gbs * 1e9), d2h / (d2h_gbs * 1e9), (h2d + d2h) / (dup_gbs * 1e9))
    del host, dev, host2, dev2
    return {"h2d_gbs": round(h2d_gbs, 1), "d2h_gbs": round(d2h_gbs, 1), "duplex_gbs": round(dup_gbs, 1),
            "step_floor_ms": round(floor_s * 1e3, 3), "frac_of_link": round(floor_s / step_s, 3)}


def run_agg(args, omg, torch, dev, stream, barrier, max_over_ranks, world):
    """Uniform-key HashAggregation over 2^22 device-resident rows."""
    L, D = omg.LongType(), omg.DoubleType()
    key, v1, v2 = agg_data_numpy(2)
    tk = torch.from_numpy(key).to(dev)
    t1 = torch.from_numpy(v1).to(dev)
    t2 = torch.from_numpy(v2).to(dev)
    flush = torch.empty(1 << 27, dtype=torch.int32, device=dev)  # 512 MB > L2
    fac = omg.HashAggregationOperatorFactory(
        [0], [L], [[1], [1], [1], [1], [2], [2]], [[L], [L], [L], [L], [D], [D]], [[L], [L], [L], [L], [D], [D]],
        [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN, omg.OMNI_AGGREGATION_TYPE_MIN,
         omg.OMNI_AGGREGATION_TYPE_MAX, omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_AVG])

    def step():
        op = fac.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        op.add_input(omg.wrap_device_batch([L, L, D], AGG_ROWS, [tk.data_ptr(), t1.data_ptr(), t2.data_ptr()]))
        groups = 0
        for b in op.drain():
            groups += omg.batch_row_count(b)
            omg.free_batch(b)
        c = op.counters()
        op.delete()
        return groups, c

    for _ in range(args.warmup):
        flush.fill_(1)
        assert step()[0] == AGG_GROUPS
    tot_ms = kern_ns = 0.0
    launches = 0
    for _ in range(args.steps):
        flush.fill_(1)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        groups, c = step()
        e1.record(stream)
        barrier()
        tot_ms += e0.elapsed_time(e1)
        kern_ns += c["kernel_ns"] / max(c["kernel_launches"], 1)
        launches += c["launches"]
        assert groups == AGG_GROUPS
    ms = max_over_ranks(tot_ms) / args.steps
    kernel_s = kern_ns / args.steps / 1e9
    alg = AGG_ROWS * 24 + AGG_GROUPS * 56
    peak, kind = measured_peak_gbs()
    traffic_per_row = profiled_traffic("agg_partitioned_kernel_agg2e22.md")
    # Parity at full size (outside the timed steps): one more operator over the same rows with
    # host output, every group against the oracle.
    op = fac.create_operator()
    op.set_stream(stream.cuda_stream)
    op.add_input(omg.wrap_device_batch([L, L, D], AGG_ROWS, [tk.data_ptr(), t1.data_ptr(), t2.data_ptr()]))
    gpu_cols = host_columns(omg, op.drain())
    op.delete()
    fac.close()
    check = check_agg_uniform(key, v1, v2, gpu_cols)
    return {"value": world * AGG_ROWS / (ms / 1e3), "unit": "rows/s", "ms_per_step": ms, "gpu_launches": launches,
            "oracle_check": check, "oracle_match": check["oracle_match"],
            "workload": "hash aggregation: 2^22 rows, int64 key over 10,000 values, SUM/COUNT/MIN/MAX(int64), "
                        "SUM/AVG(double); input resident in HBM, L2 flushed between steps",
            "roofline": {"bound": "hbm", "achieved": round(alg / kernel_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(alg / kernel_s / 1e9 / peak, 4), "peak_kind": kind,
                         "traffic": None if traffic_per_row is None else round(traffic_per_row * AGG_ROWS),
                         "kernel": "AggPartKernel", "kernel_ms": round(kernel_s * 1e3, 4),
                         "algorithmic_bytes": alg}}


def check_agg_uniform(key, v1, v2, gpu_cols):
    """The uniform aggregation's GPU groups against the oracle (all rows, all groups)."""
    import oracle

    oracle.build()
    aggs = [dict(func=f, col=v1, in_type=oracle.T_LONG, out_type=oracle.T_LONG)
            for f in (oracle.F_SUM, oracle.F_COUNT_COL, oracle.F_MIN, oracle.F_MAX)]
    aggs += [dict(func=oracle.F_SUM, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE),
             dict(func=oracle.F_AVG, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE),
             dict(func=oracle.F_COUNT_COL, col=v2, in_type=oracle.T_DOUBLE, out_type=oracle.T_LONG)]
    t0 = time.perf_counter()
    ora = oracle.hashagg_mt([key], [oracle.T_LONG], [None], aggs, threads=host_threads())
    res = compare_agg_full(gpu_cols, ora, 1, {4: (4, None), 5: (5, 6)})
    res["check_s"] = round(time.perf_counter() - t0, 2)
    res["rows"] = len(key)
    return res


SKEW_ROWS = 1 << 28
SKEW_PAIRS = 50_000_000
SKEW_WORKLOAD = ("hash aggregation, high-cardinality skewed: 2^28 rows, key (int32, int64) pair of Zipf(1.1) "
                 "rank over 50,000,000 pairs; SUM(decimal64(18,2) uniform unscaled [-1e9, 1e9]) -> "
                 "decimal128(38,2), COUNT(*), AVG(double N(0,1)); 2% NULLs per value column; input resident in "
                 "HBM (7.6 GB, larger than L2)")


def nulls_bitmap(torch, mask):
    """LSB-first validity bitmap (set bit = NULL) of a bool tensor, padded to whole words."""
    n = mask.numel()
    pad = (-n) % 64
    m = torch.cat([mask, torch.zeros(pad + 64, dtype=torch.bool, device=mask.device)])
    weights = torch.tensor([1, 2, 4, 8, 16, 32, 64, 128], device=mask.device, dtype=torch.int32)
    return (m.view(-1, 8).to(torch.int32) * weights).sum(1).to(torch.uint8)


def run_agg_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank):
    """Plain vs learned sizing on the skewed high-cardinality aggregation (one operator per step)."""
    from omnioperator_gb300 import sizer, sizer_train

    I, L, D = omg.IntType(), omg.LongType(), omg.DoubleType()
    d64, d128 = omg.Decimal64Type(18, 2), omg.Decimal128Type(38, 2)
    g = torch.Generator(device=dev)
    g.manual_seed(4242 + rank)
    n = SKEW_ROWS if args.skew_log2 is None else 1 << args.skew_log2
    cdf = sizer_train.zipf_cdf(torch, SKEW_PAIRS, 1.1, dev)
    rank_ = torch.empty(n, dtype=torch.int64, device=dev)
    chunk = 1 << 25
    for s0 in range(0, n, chunk):
        u = torch.rand(min(chunk, n - s0), generator=g, device=dev, dtype=torch.float64)
        rank_[s0:s0 + len(u)] = torch.searchsorted(cdf, u).clamp_(max=SKEW_PAIRS - 1)
    del cdf
    k1 = (rank_ % 65521).to(torch.int32)
    x = rank_ * 0x100000001B3 + 7
    x = x ^ ((x >> 30) & 0x3FFFFFFFF)
    x = x * -4658895280553007687
    x = x ^ ((x >> 27) & 0x1FFFFFFFFF)
    x = x * -7723592293110705685
    k2 = x ^ ((x >> 31) & 0x1FFFFFFFF)
    del x, rank_
    dec = torch.randint(-10**9, 10**9 + 1, (n,), generator=g, device=dev, dtype=torch.int64)
    dbl = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
    dec_nulls = nulls_bitmap(torch, torch.rand(n, generator=g, device=dev) < 0.02)
    dbl_nulls = nulls_bitmap(torch, torch.rand(n, generator=g, device=dev) < 0.02)
    torch.cuda.synchronize()

    model_path = Path(args.sizer) if args.sizer else ROOT / "omnioperator_gb300" / "models" / "agg_sizer.json"
    if model_path.exists():
        model = sizer.SizingModel.load(str(model_path))
        model_src = str(model_path.relative_to(ROOT)) if model_path.is_relative_to(ROOT) else str(model_path)
    else:  # no trained weights shipped: train on the plain operator's records now
        recs = sizer_train.collect(torch, 48, 99, n_max=1 << 26, log=None)
        model, _ = sizer_train.train(recs, epochs=3000)
        model_src = "trained at bench start on 48 plain-operator records"

    def factory(arm):
        f = omg.HashAggregationOperatorFactory(
            [0, 1], [I, L], [[2], [], [3]], [[d64], [], [D]], [[d128], [L], [D]],
            [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_ALL, omg.OMNI_AGGREGATION_TYPE_AVG])
        if arm == "learned":
            f.set_sizer(model)
        return f

    hint = {}

    def step(fac):
        op = fac.create_operator()
        if hint.get("groups"):
            op.set_agg_strategy(omg.AGG_STRATEGY_AUTO, hint["groups"])
        if hint.get("hll"):
            op.set_agg_sizing(omg.AGG_SIZING_HLL)
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        op.add_input(omg.wrap_device_batch([I, L, d64, D], n, [k1.data_ptr(), k2.data_ptr(), dec.data_ptr(),
                                                              dbl.data_ptr()],
                                           [None, None, dec_nulls.data_ptr(), dbl_nulls.data_ptr()]))
        outs, groups = op.get_outputs(1 << 16)
        omg.free_batches(outs)
        c = op.counters()
        slog = op.sizing_log()
        op.delete()
        return groups, c, slog

    steps = max(1, min(args.steps, 3))
    res = {}
    # exact_count: the true group count given as the capacity hint (the best any estimate can do);
    # hll: a HyperLogLog sketch of every row's key (a distinct-count sketch, the competent
    # non-learned estimate; its extra pass over the keys is inside the timed step).
    for arm in ("plain", "learned", "hll", "exact_count"):
        fac = factory(arm)
        hint.clear()
        if arm == "exact_count":
            hint["groups"] = res["plain"]["groups"]
        if arm == "hll":
            hint["hll"] = True
        step(fac)  # warm-up
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            groups, c, slog = step(fac)
        e1.record(stream)
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1)) / steps
        fac.close()
        res[arm] = {"value": world * n / (ms / 1e3), "unit": "rows/s", "ms_per_step": round(ms, 3),
                    "kernel_s": c["kernel_ns"] / max(c["kernel_launches"], 1) / 1e9,
                    "groups": groups, "estimate": slog["estimate"], "plain_estimate": slog["plain_estimate"],
                    "table_resizes": c["resizes"], "retried_rows": c["retried_rows"],
                    "shared_front_table": slog["smem_front"], "part_bits": slog["part_bits"]}
    assert res["plain"]["groups"] == res["learned"]["groups"] == res["exact_count"]["groups"] == res["hll"]["groups"]
    # Roofline of the aggregation kernel (the learned arm's launches): 28.25 B read per row
    # (4 + 8 + 8 + 8 B and two validity bits), 45 B written per group.
    groups = res["learned"]["groups"]
    alg = n * 28.25 + groups * 45
    peak, kind = measured_peak_gbs()
    for arm in res:
        res[arm]["kernel_ms"] = round(res[arm].pop("kernel_s") * 1e3, 3)
    kern_s = res["learned"]["kernel_ms"] / 1e3
    roofline = {"bound": "hbm", "achieved": round(alg / kern_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                "frac": round(alg / kern_s / 1e9 / peak, 4), "peak_kind": kind, "traffic": None,
                "kernel": "AggKernel (global table)", "kernel_ms": round(kern_s * 1e3, 3), "algorithmic_bytes": int(alg)}
    # Parity at full size (outside the timed steps): the learned operator's groups, with host
    # output, against the oracle over every row.
    fac = factory("learned")
    op = fac.create_operator()
    op.set_stream(stream.cuda_stream)
    op.add_input(omg.wrap_device_batch([I, L, d64, D], n, [k1.data_ptr(), k2.data_ptr(), dec.data_ptr(),
                                                          dbl.data_ptr()],
                                       [None, None, dec_nulls.data_ptr(), dbl_nulls.data_ptr()]))
    gpu_cols = host_columns(omg, op.drain())
    op.delete()
    fac.close()
    model.close()

    # All rows when the host has room for them and the oracle's tables, else the rows of one
    # eighth of the groups (k2 mod 8 == 0; k2 identifies the pair) against the same GPU groups.
    need = n * 40 + groups * 400
    avail = mem_available_bytes()
    sel = None
    if avail is not None and avail < 2 * need:
        sel = (k2 & 7) == 0
        keep = ~((gpu_cols[1][0] & 7).astype(bool))
        gpu_cols = [(v[keep], m[keep]) for v, m in gpu_cols]
        groups = len(gpu_cols[0][0])

    def host(t):
        return (t[sel] if sel is not None else t).cpu().numpy()

    def unbits(t):
        m = torch.from_numpy(np.unpackbits(t.cpu().numpy(), bitorder="little")[:n].astype(bool))
        return (m[sel.cpu()] if sel is not None else m).numpy()

    log("skewed aggregation timed; oracle check")
    check, cpu = check_agg_skewed(host(k1), host(k2), host(dec), host(dbl), unbits(dec_nulls), unbits(dbl_nulls),
                                  gpu_cols, groups)
    check["scope"] = "all rows" if sel is None else "rows of the groups with k2 mod 8 == 0 (host memory)"
    return {"workload": SKEW_WORKLOAD if n == SKEW_ROWS else SKEW_WORKLOAD.replace("2^28", f"2^{n.bit_length() - 1}"),
            "steps": steps, "sizer": model_src, "plain": res["plain"], "learned": res["learned"], "hll": res["hll"],
            "exact_count": res["exact_count"],
            "learned_over_plain": round(res["learned"]["value"] / res["plain"]["value"], 3),
            "learned_over_hll": round(res["learned"]["value"] / res["hll"]["value"], 3),
            "roofline": roofline, "cpu_baseline": cpu, "oracle_check": check, "oracle_match": check["oracle_match"]}


def check_agg_skewed(k1, k2, dec, dbl, dec_null, dbl_null, gpu_cols, groups):
    """The skewed aggregation's GPU groups against the oracle over every row (SUM(decimal64) ->
    decimal128 and COUNT(*) bit-exact, AVG(double) within 1e-12 * max(|exact|, sum|x|) / count);
    the oracle run, on all host threads, is also the CPU baseline."""
    import oracle

    oracle.build()
    aggs = [dict(func=oracle.F_SUM, col=dec, in_type=oracle.T_DEC64, out_type=oracle.T_DEC128, nulls=dec_null),
            dict(func=oracle.F_COUNT_ALL, col=None, in_type=oracle.T_LONG, out_type=oracle.T_LONG),
            dict(func=oracle.F_AVG, col=dbl, in_type=oracle.T_DOUBLE, out_type=oracle.T_DOUBLE, nulls=dbl_null),
            dict(func=oracle.F_COUNT_COL, col=dbl, in_type=oracle.T_DOUBLE, out_type=oracle.T_LONG, nulls=dbl_null)]
    threads = host_threads()
    t0 = time.perf_counter()
    ora = oracle.hashagg_mt([k1, k2], [oracle.T_INT, oracle.T_LONG], [None, None], aggs, threads=threads,
                            max_groups=max(2 * groups, 1 << 20))
    secs = time.perf_counter() - t0
    res = compare_agg_full(gpu_cols, ora, 2, {2: (2, 3)})
    res["check_s"] = round(time.perf_counter() - t0, 2)
    res["rows"] = len(k1)
    cpu = {"value": len(k1) / secs, "unit": "rows/s", "cores": threads, "kind": "port",
           "sample": f"all {len(k1)} rows, {threads} threads (rows split by key hash, each group folded in row "
                     "order by one thread; includes the double-double check sums)"}
    return res, cpu


JOIN5_BUILD = 1 << 26
JOIN5_PROBE = 1 << 30
JOIN5_WORKLOAD = ("skewed inner hash join: build 2^26 rows, key 2u for distinct u < 2^39, 16-byte payload (two int64); "
                  "probe 2^30 rows, 90% a build key of Zipf(s) rank through a seeded rank->key permutation, 10% odd "
                  "keys (no match); output (probe key, payload); 4096 partitions: direct probe vs hash partitioning "
                  "vs learned range partitioning")


def _bij39(x):
    """A bijection on [0, 2^39) (odd multiplies and an xor-shift, all mod 2^39)."""
    m = (1 << 39) - 1
    x = (x * 0x9E3779B1) & m
    x = x ^ (x >> 19)
    return (x * 0x85EBCA77) & m


def run_join_skewed(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank):
    """cfg 5: one build, three probe distributions, three probe strategies; every strategy's output
    must have the same row-multiset fingerprint as the direct probe's."""
    from omnioperator_gb300 import sizer_train

    L = omg.LongType()
    nb = JOIN5_BUILD if args.join5_build_log2 is None else 1 << args.join5_build_log2
    npb = JOIN5_PROBE if args.join5_probe_log2 is None else 1 << args.join5_probe_log2
    g = torch.Generator(device=dev)
    g.manual_seed(5150 + rank)
    idx = torch.arange(nb, device=dev, dtype=torch.int64)
    bkey = 2 * _bij39(idx)
    pay1 = torch.randint(-2**62, 2**62, (nb,), generator=g, device=dev, dtype=torch.int64)
    pay2 = torch.randint(-2**62, 2**62, (nb,), generator=g, device=dev, dtype=torch.int64)
    bf = omg.HashBuilderOperatorFactory(omg.OMNI_JOIN_TYPE_INNER, [L, L, L], [0])
    bop = bf.create_operator()
    bop.set_stream(stream.cuda_stream)
    bop.add_input(omg.wrap_device_batch([L, L, L], nb, [bkey.data_ptr(), pay1.data_ptr(), pay2.data_ptr()]))
    bop.get_output()
    pf = omg.LookupJoinOperatorFactory([L], [0], [0], [1, 2], [L, L], bf)
    steps = max(1, min(args.steps, 3))
    bits = 12
    out = {"workload": JOIN5_WORKLOAD, "build_rows": nb, "probe_rows": npb, "partitions": 1 << bits, "steps": steps}
    import oracle

    oracle.build()
    t0 = time.perf_counter()
    bkey_h, pay_h = bkey.cpu().numpy(), [pay1.cpu().numpy(), pay2.cpu().numpy()]
    jt = oracle.JoinTable(bkey_h)
    out["oracle_build_s"] = round(time.perf_counter() - t0, 2)
    peak, peak_kind = measured_peak_gbs()
    for s in (0.9, 1.1, 1.3):
        cdf = sizer_train.zipf_cdf(torch, nb, s, dev)
        pkey = torch.empty(npb, dtype=torch.int64, device=dev)
        chunk = 1 << 26
        for s0 in range(0, npb, chunk):
            m = min(chunk, npb - s0)
            r = torch.searchsorted(cdf, torch.rand(m, generator=g, device=dev, dtype=torch.float64)).clamp_(max=nb - 1)
            hit = bkey[(r * 0x9E3779B1) & (nb - 1)]  # rank -> build row (odd multiply mod 2^26)
            miss = 2 * torch.randint(0, 1 << 39, (m,), generator=g, device=dev, dtype=torch.int64) + 1
            pkey[s0:s0 + m] = torch.where(torch.rand(m, generator=g, device=dev) < 0.9, hit, miss)
        del cdf
        torch.cuda.synchronize()
        sample = pkey[:: max(1, npb // 65536)].cpu().numpy()
        t0 = time.perf_counter()
        splits = omg.learn_splits(sample, bits=bits, epochs=2000)
        learn_ms = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        qsplits = omg.quantile_splits(sample, bits=bits)  # the method without a network
        quantile_ms = (time.perf_counter() - t0) * 1e3
        per = {}
        chosen = {}
        gpu_fp = {}
        for name, strat in (("direct", omg.JOIN_DIRECT), ("hash_partitioned", omg.JOIN_HASH_PARTITIONED),
                            ("learned_range_partitioned", omg.JOIN_RANGE_PARTITIONED),
                            ("learned_choice", omg.JOIN_LEARNED), ("quantile_choice", omg.JOIN_QUANTILE)):
            def step(fp=False):
                op = pf.create_operator()
                op.set_stream(stream.cuda_stream)
                op.set_device_output(True)
                op.set_join_strategy(strat, bits,
                                     splits if strat in (omg.JOIN_RANGE_PARTITIONED, omg.JOIN_LEARNED) else
                                     (qsplits if strat == omg.JOIN_QUANTILE else None))
                chosen[name] = op.join_strategy()
                op.add_input(omg.wrap_device_batch([L], npb, [pkey.data_ptr()]))
                outs, rows = op.get_outputs(1 << 20)
                f = omg.batches_fingerprint(outs) if fp else None
                omg.free_batches(outs)
                kern[name] = op.counters()
                op.delete()
                return rows, f
            kern = {}
            rows, fp = step(fp=True)  # warm-up (also builds the partitioned build tables) + fingerprint
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                step()
            e1.record(stream)
            barrier()
            ms = max_over_ranks(e0.elapsed_time(e1)) / steps
            c = kern[name]
            dev_ms = c["kernel_ns"] / max(c["kernel_launches"], 1) / 1e6
            per[name] = {"value": world * npb / (ms / 1e3), "unit": "rows/s", "ms_per_step": round(ms, 2),
                         "device_ms": round(dev_ms, 2), "output_rows": rows,
                         "fingerprint": f"{fp[1]:016x}{fp[2]:016x}"}
            gpu_fp[name] = fp
        ref = per["direct"]["fingerprint"]
        assert all(v["fingerprint"] == ref and v["output_rows"] == per["direct"]["output_rows"] for v in per.values())
        log(f"skewed join s={s} timed; oracle check")
        # Parity at full size (outside the timed steps): the output's fingerprint against the
        # oracle's join of all 2^30 probe rows (probed in chunks; the fingerprint is a sum), and
        # the exact rows of the probe keys with (key >> 1) mod 64 == 0 against the oracle's.
        t0 = time.perf_counter()
        ofp, osecs = [0, 0, 0], 0.0
        for c0 in range(0, npb, 1 << 27):
            f, sec = jt.fingerprint(pay_h, pkey[c0:c0 + (1 << 27)].cpu().numpy(), None, threads=host_threads())
            ofp = [(a + b) & ((1 << 64) - 1) for a, b in zip(ofp, f)]
            osecs += sec
        fp_match = all(tuple(v) == tuple(ofp) for v in gpu_fp.values())
        slice_keys = pkey[((pkey >> 1) & 63) == 0].contiguous()
        op = pf.create_operator()
        op.set_stream(stream.cuda_stream)
        op.add_input(omg.wrap_device_batch([L], len(slice_keys), [slice_keys.data_ptr()]))
        gcols = host_columns(omg, op.drain())
        op.delete()
        sk = slice_keys.cpu().numpy()
        pi, bi = jt.pairs(sk)
        ocols = [sk[pi], pay_h[0][bi], pay_h[1][bi]]
        if gcols is None:
            slice_match = len(pi) == 0
        else:
            go, oo = np.argsort(gcols[0][0], kind="stable"), np.argsort(ocols[0], kind="stable")
            slice_match = len(go) == len(oo) and all(
                np.array_equal(g[0][go], o[oo]) and not g[1].any() for g, o in zip(gcols, ocols))
        del slice_keys
        per["oracle_check"] = {"oracle_match": bool(fp_match and slice_match), "fingerprint_match": fp_match,
                               "rows": int(ofp[0]), "slice_rows": int(len(pi)), "slice_match": bool(slice_match),
                               "check_s": round(time.perf_counter() - t0, 2)}
        per["cpu_baseline"] = {"value": npb / osecs, "unit": "rows/s", "cores": host_threads(), "kind": "port",
                               "sample": f"all {npb} probe rows against the 2^26-row build, "
                                         f"{host_threads()} threads, output rows hashed (not materialised)"}
        best = min(("direct", "hash_partitioned", "learned_range_partitioned", "learned_choice", "quantile_choice"),
                   key=lambda k: per[k]["device_ms"])
        alg = npb * 8 + per["direct"]["output_rows"] * 24
        dev_s = per["learned_choice"]["device_ms"] / 1e3
        per["roofline"] = {"bound": "hbm", "achieved": round(alg / dev_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                           "frac": round(alg / dev_s / 1e9 / peak, 4), "peak_kind": peak_kind, "traffic": None,
                           "kernel": "learned choice's device time (partition passes + probes, or the direct probe)",
                           "kernel_ms": round(dev_s * 1e3, 3), "algorithmic_bytes": int(alg),
                           "fastest_strategy": best}
        top = float(cdf_top_share(torch, nb, s, dev))
        per["learned_choice"]["strategy"] = {0: "direct", 1: "hash_partitioned", 2: "range_partitioned"}[
            chosen["learned_choice"]]
        per["quantile_choice"]["strategy"] = {0: "direct", 1: "hash_partitioned", 2: "range_partitioned"}[
            chosen["quantile_choice"]]
        per["splits_learn_ms"] = round(learn_ms, 1)
        per["splits_quantile_ms"] = round(quantile_ms, 2)
        # One query pays its split learning: the learned choice's time with it included.
        per["learned_choice"]["ms_incl_learning"] = round(per["learned_choice"]["ms_per_step"] + learn_ms, 1)
        per["quantile_choice"]["ms_incl_splits"] = round(per["quantile_choice"]["ms_per_step"] + quantile_ms, 2)
        per["top_key_share"] = round(top, 4)
        out[f"s={s}"] = per
        del pkey
    jt.close()
    out["oracle_match"] = all(out[f"s={s}"]["oracle_check"]["oracle_match"] for s in (0.9, 1.1, 1.3))
    pf.close()
    bop.delete()
    bf.close()
    return out


def cdf_top_share(torch, n, s, dev):
    w = torch.arange(1, n + 1, device=dev, dtype=torch.float64).pow_(-s)
    return 0.9 * (w[0] / w.sum()).item()


BATCH_TASKS = 10_000
BATCH_WORKLOAD = ("batched small aggregations: 10,000 independent tasks, rows per task log-uniform [1e3, 1e6], "
                  "int64 key uniform over a per-task domain log-uniform [10, min(rows, 1e6)], SUM and COUNT of an "
                  "int64 value; inputs resident in HBM (one batch per task)")


def run_agg_batched(args, omg, torch, dev, stream, barrier, max_over_ranks, world, rank):
    """10,000 tasks: one operator per task (sample) vs one batched launch, plain and learned sizing."""
    from omnioperator_gb300 import sizer, sizer_train

    L = omg.LongType()
    n_tasks = BATCH_TASKS if args.batch_tasks is None else args.batch_tasks
    keys, vals, spans = sizer_train.make_tasks(torch, n_tasks, 77 + rank, dev)
    torch.cuda.synchronize()
    total_rows = sum(n for _, n in spans)

    def factory():
        return omg.HashAggregationOperatorFactory(
            [0], [L], [[1], [1]], [[L], [L]], [[L], [L]],
            [omg.OMNI_AGGREGATION_TYPE_SUM, omg.OMNI_AGGREGATION_TYPE_COUNT_COLUMN])

    def views():
        return [omg.wrap_device_batch([L, L], n, [keys.data_ptr() + 8 * o, vals.data_ptr() + 8 * o]) for o, n in spans]

    res = {}
    # One operator per task (the reference's structure), on a bounded sample of the tasks.
    sample = spans[: max(1, min(len(spans), args.batch_operator_sample))]
    fac = factory()
    barrier()
    t0 = time.perf_counter()
    groups_sample = 0
    for o, n in sample:
        op = fac.create_operator()
        op.set_stream(stream.cuda_stream)
        op.set_device_output(True)
        op.add_input(omg.wrap_device_batch([L, L], n, [keys.data_ptr() + 8 * o, vals.data_ptr() + 8 * o]))
        outs, g = op.get_outputs(1 << 12)
        groups_sample += g
        omg.free_batches(outs)
        op.delete()
    barrier()
    dt = max_over_ranks(time.perf_counter() - t0)
    fac.close()
    sample_rows = sum(n for _, n in sample)
    res["operators"] = {"value": world * sample_rows / dt, "unit": "rows/s", "tasks": len(sample),
                        "rows": sample_rows, "ms": round(dt * 1e3, 2)}

    model_path = ROOT / "omnioperator_gb300" / "models" / "agg_task_sizer.json"
    model = sizer.SizingModel.load(str(model_path)) if model_path.exists() else None
    steps = max(1, min(args.steps, 5))
    for arm in ("batched_plain", "batched_learned"):
        if arm == "batched_learned" and model is None:
            continue
        fac = factory()
        handles = views()
        b = omg.AggBatch(fac, handles, sizer=model if arm == "batched_learned" else None,
                         flags=omg.BATCH_DEVICE_OUTPUT)
        barrier()
        t0 = time.perf_counter()
        b.run(stream.cuda_stream)  # sizing, tuning, graph capture, first run
        outs = b.outputs()
        omg.free_batches([x for _, x in outs])
        first_ms = (time.perf_counter() - t0) * 1e3
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        for _ in range(steps):
            b.run(stream.cuda_stream)  # graph replay
            outs = b.outputs()
            omg.free_batches([x for _, x in outs])
        e1.record(stream)
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1)) / steps
        info = b.info()
        if arm == "batched_learned" or model is None:
            # Parity (outside the timed runs): one more run, a sample of the tasks' outputs
            # against the oracle's per-task aggregation of the same rows.
            log(f"batched {arm} timed; oracle check")
            b.run(stream.cuda_stream)
            outs = b.outputs()
            check, cpu = check_tasks(omg, keys, vals, spans, outs, args.batch_check_every)
            omg.free_batches([x for _, x in outs])
            res["oracle_check"] = check
            res["cpu_baseline"] = cpu
        b.close()
        omg.free_batches(handles)
        fac.close()
        res[arm] = {"value": world * total_rows / (ms / 1e3), "unit": "rows/s", "ms_per_step": round(ms, 3),
                    "first_run_ms": round(first_ms, 1), "groups": info["groups"], "table_slots": info["table_slots"],
                    "tasks_rerun_exactly": info["reruns"], "tasks_grown_batched": info.get("grown"),
                    "tasks_rerun_by_operator": info.get("operator_reruns"), "threads": info["threads"],
                    "ctas_per_sm": info["ctas_per_sm"], "graph": bool(info["graph"]), "tune_ms": info["tune_us"] / 1e3,
                    "device_ms": info["run_us"] / 1e3}
    if model is not None:
        model.close()
    arm = res.get("batched_learned", res.get("batched_plain"))
    if arm is not None:
        alg = total_rows * 16 + arm["groups"] * 24
        dev_s = arm["device_ms"] / 1e3
        peak, kind = measured_peak_gbs()
        res["roofline"] = {"bound": "hbm", "achieved": round(alg / dev_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                           "frac": round(alg / dev_s / 1e9 / peak, 4), "peak_kind": kind, "traffic": None,
                           "kernel": "the batched launch (graph: table init, AggTasksKernel, counts, extraction)",
                           "kernel_ms": round(dev_s * 1e3, 3), "algorithmic_bytes": int(alg)}
    out = {"workload": BATCH_WORKLOAD if n_tasks == BATCH_TASKS else BATCH_WORKLOAD.replace("10,000", str(n_tasks)),
           "tasks": n_tasks, "rows": total_rows, "steps": steps, **res}
    if "oracle_check" in res:
        out["oracle_match"] = res["oracle_check"]["oracle_match"]
    if "batched_plain" in res:
        out["batched_over_operators"] = round(res["batched_plain"]["value"] / res["operators"]["value"], 2)
    if "batched_learned" in res:
        out["learned_over_plain"] = round(res["batched_learned"]["value"] / res["batched_plain"]["value"], 3)
    return out


def check_tasks(omg, keys, vals, spans, outs, every):
    """Every `every`-th task of a batched run against the oracle: the task's output rows (key,
    SUM, COUNT) fingerprinted on the GPU against the fingerprint of the oracle's aggregation of
    the task's rows (groups and values bit-exact).  The oracle runs one task per host thread;
    its rate is the CPU baseline."""
    import concurrent.futures as cf

    import oracle

    oracle.build()
    by_task = {}
    for t, bh in outs:
        by_task.setdefault(t, []).append(bh)
    picked = list(range(0, len(spans), max(1, every)))
    threads = host_threads()
    host_keys = {t: (keys[spans[t][0]:spans[t][0] + spans[t][1]].cpu().numpy(),
                     vals[spans[t][0]:spans[t][0] + spans[t][1]].cpu().numpy()) for t in picked}

    def one(t):
        k, v = host_keys[t]
        aggs = [dict(func=f, col=v, in_type=oracle.T_LONG, out_type=oracle.T_LONG)
                for f in (oracle.F_SUM, oracle.F_COUNT_COL)]
        t0 = time.perf_counter()
        ks, kn, vs, vn = oracle.hashagg([k], [oracle.T_LONG], [None], aggs)
        dt = time.perf_counter() - t0
        return oracle.fingerprint_cols([ks[0], vs[0], vs[1]], [kn[0], vn[0], vn[1]]), len(k), dt

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        results = list(ex.map(one, picked))
    wall = time.perf_counter() - t0
    bad = []
    for t, (fp, _, _) in zip(picked, results):
        gfp = omg.batches_fingerprint(by_task.get(t, []))
        if tuple(gfp) != tuple(fp):
            bad.append(t)
    rows = sum(n for _, n, _ in results)
    cpu_s = sum(dt for _, _, dt in results)
    check = {"oracle_match": not bad, "tasks_checked": len(picked), "rows_checked": rows,
             "mismatched_tasks": bad[:8], "check_s": round(wall, 2)}
    cpu = {"value": rows / (cpu_s / threads), "unit": "rows/s", "cores": threads, "kind": "port",
           "sample": f"{len(picked)} of {len(spans)} tasks ({rows} rows), one single-threaded operator per task; "
                     f"rate = rows / (sum of per-task seconds / {threads} threads)"}
    return check, cpu


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-agg", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "agg", "skew", "batched", "join5"],
                    help="agg / skew: time only that aggregation workload (profiling runs)")
    ap.add_argument("--probe-log2", type=int, default=26, help="log2 of probe rows (profiling runs use fewer)")
    ap.add_argument("--bulk-probe", type=int, default=0, choices=[0, 1, 2],
                    help="headline probe kernel: 0 per-lane bitmap kernel, 1 bulk-copy key loads, "
                         "2 bulk-copy key loads and output stores")
    ap.add_argument("--skip-skew", action="store_true", help="skip the skewed aggregation (plain vs learned)")
    ap.add_argument("--skew-log2", type=int, default=None, help="log2 rows of the skewed aggregation (default 28)")
    ap.add_argument("--sizer", default=None, help="sizing model weights (JSON) for the learned arm")
    ap.add_argument("--skip-batched", action="store_true", help="skip the batched small aggregations")
    ap.add_argument("--skip-join5", action="store_true", help="skip the skewed join (partitioners)")
    ap.add_argument("--skip-ext", action="store_true",
                    help="skip the other join kinds and the two-stage aggregation")
    ap.add_argument("--join5-build-log2", type=int, default=None)
    ap.add_argument("--join5-probe-log2", type=int, default=None)
    ap.add_argument("--batch-tasks", type=int, default=None, help="tasks of the batched aggregation (default 10,000)")
    ap.add_argument("--batch-operator-sample", type=int, default=500,
                    help="tasks run one operator each for the per-operator comparison")
    ap.add_argument("--batch-check-every", type=int, default=10,
                    help="every n-th task of the batched run is checked against the oracle")
    args = ap.parse_args()
    global N_PROBE
    N_PROBE = 1 << args.probe_log2
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    r = run_gpu(args, rank, world)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        import oracle

        oracle.build()
        threads = os.cpu_count() or 1
        data = join_data_numpy(1, n_probe=1 << 24)
        v = cpu_join_rows_per_s(data, threads, reps=3)
        cpu = {"value": v, "unit": "rows/s", "cores": threads, "kind": "port",
               "sample": f"build 2^20 + probe 2^24 of the 2^26 probe rows, {threads} threads, median of 3"}
        if r["agg"] is not None:
            r["agg"]["cpu_baseline"] = {"value": cpu_agg_rows_per_s(agg_data_numpy(2), threads, reps=3),
                                        "unit": "rows/s", "cores": threads, "kind": "port",
                                        "sample": "full 2^22-row workload, partial per thread + final merge"}
    line = base_line(args, r["value"], r["ms"])
    line.update({"config": {"workload": JOIN_WORKLOAD, "step": "LookupJoin over the 2^26 probe rows, build resident",
                            "l2": "inputs+outputs (1.4 GB/step) larger than L2; no flush needed",
                            "build_ms": round(r["build_ms"], 3), "output_rows_per_step": r["rows"]},
                 "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r["e2e"], "gpu_launches": r["launches"],
                 "clocks": r["clocks"], "oracle_match": None if r.get("join_check") is None else
                 r["join_check"]["oracle_match"], "oracle_check": r.get("join_check"),
                 "agg": r["agg"], "agg_skewed": r["skew"], "agg_batched": r["batched"],
                 "join_skewed": r["join5"], "join_kinds": r.get("kinds"), "agg_two_stage": r.get("two_stage"),
                 "features": r.get("features")})
    line["summary"] = summary(line)  # last key: a compact per-configuration digest
    print(json.dumps(line), flush=True)


def _sig(x, d=3):
    """x rounded to d significant digits (None stays None)."""
    if x is None:
        return None
    if x == 0:
        return 0
    return float(f"{x:.{d}g}")


def summary(line):
    """One short object per configuration (rows/s, ms, roofline fraction, CPU baseline, oracle
    verdict), placed at the end of the JSON line so that a reader of its tail sees them all."""
    out = {}
    e2e = line.get("e2e") or {}
    cpu = line.get("cpu_baseline") or {}
    out["cfg2_probe"] = {"rows_s": _sig(line["value"]), "ms": _sig(line["ms_per_step"]),
                         "frac": (line.get("roofline") or {}).get("frac"), "e2e_rows_s": _sig(e2e.get("value")),
                         "e2e_ms": _sig(e2e.get("ms_per_step")), "e2e_link_frac": (e2e.get("link") or {}).get("frac_of_link"),
                         "cpu_rows_s": _sig(cpu.get("value")),
                         "oracle_match": line.get("oracle_match"), "e2e_oracle_match": e2e.get("oracle_match")}
    a = line.get("agg")
    if a:
        out["cfg1_agg"] = {"rows_s": _sig(a["value"]), "ms": _sig(a["ms_per_step"]), "frac": a["roofline"]["frac"],
                           "kernel_ms": a["roofline"]["kernel_ms"],
                           "cpu_rows_s": _sig((a.get("cpu_baseline") or {}).get("value")),
                           "oracle_match": a.get("oracle_match")}
    k = line.get("agg_skewed")
    if k:
        out["cfg3_skew"] = {"plain_ms": k["plain"]["ms_per_step"], "learned_ms": k["learned"]["ms_per_step"],
                            "hll_ms": k["hll"]["ms_per_step"],
                            "exact_count_ms": k["exact_count"]["ms_per_step"],
                            "learned_over_plain": k["learned_over_plain"], "frac": k["roofline"]["frac"],
                            "cpu_rows_s": _sig(k["cpu_baseline"]["value"]), "oracle_match": k.get("oracle_match")}
    b = line.get("agg_batched")
    if b:
        out["cfg4_batched"] = {"operators_rows_s": _sig(b["operators"]["value"]),
                               "plain_rows_s": _sig((b.get("batched_plain") or {}).get("value")),
                               "learned_rows_s": _sig((b.get("batched_learned") or {}).get("value")),
                               "learned_over_plain": b.get("learned_over_plain"),
                               "frac": (b.get("roofline") or {}).get("frac"),
                               "cpu_rows_s": _sig((b.get("cpu_baseline") or {}).get("value")),
                               "oracle_match": b.get("oracle_match")}
    j = line.get("join_skewed")
    if j:
        d = {}
        for sk in ("s=0.9", "s=1.1", "s=1.3"):
            if sk in j:
                v = j[sk]
                d[sk] = [v["direct"]["ms_per_step"], v["hash_partitioned"]["ms_per_step"],
                         v["learned_range_partitioned"]["ms_per_step"], v["learned_choice"]["ms_per_step"],
                         v["quantile_choice"]["ms_per_step"], v["roofline"]["frac"]]
        out["cfg5_join_ms_direct_hash_range_learned_quantile_frac"] = d
        out["cfg5_cpu_rows_s"] = _sig(j["s=1.1"]["cpu_baseline"]["value"]) if "s=1.1" in j else None
        out["cfg5_oracle_match"] = j.get("oracle_match")
    kinds = line.get("join_kinds") or {}
    feats = line.get("features") or {}
    fr = {name: v["roofline"]["frac"] for name, v in kinds.items() if isinstance(v, dict) and "roofline" in v}
    if "join_filter" in feats and "roofline" in feats["join_filter"]:
        fr["filter"] = feats["join_filter"]["roofline"]["frac"]
    if fr:
        out["probe_kind_frac"] = fr
    return out


if __name__ == "__main__":
    main()
