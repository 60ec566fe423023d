"""The N > 1 path of bench.py on the CPU: two ranks over gloo (127.0.0.1).  Replicas share no data
path; they only meet at the barriers around the timed region and in the MAX over their elapsed
times, from which the whole-job rate is world x per-rank units / the slowest rank's time.  Each
rank draws its own seeded data, and the reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        barrier, max_over_ranks = bench.replica_sync(dist, torch.device("cpu"))
        barrier()
        slowest = max_over_ranks(0.25 * (rank + 1))  # rank r "took" 0.25 (r + 1) s
        barrier()
        rate = bench.whole_job_rate(world, 1000, slowest)
        key = bench.join_data_numpy(7 + rank, n_probe=4096)[3]
        (Path(out_dir) / f"rank{rank}.txt").write_text(f"{slowest} {rate} {int(key[:64].sum())}")
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [(tmp_path / f"rank{r}.txt").read_text().split() for r in range(world)]
    for slowest, rate, _ in res:
        assert float(slowest) == 0.5  # both ranks see the slowest rank's time
        assert float(rate) == world * 1000 / 0.5
    assert res[0][2] != res[1][2]  # each replica processes its own data


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""
