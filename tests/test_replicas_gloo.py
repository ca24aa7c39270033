"""The multi-rank bench path on CPU: world_size-2 gloo ranks (127.0.0.1).
Replicas share no data; the only collectives are the timing barrier and the
max over ranks, and the reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_setup()[:2] == (world, rank)
        bench.rank_barrier(world)
        q.put((rank, bench.rank_max(1.5 + rank, world, torch.device("cpu"))))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    bench.rank_barrier(1)
    assert bench.rank_max(3.25, 1, "cpu") == 3.25


def test_reference_arm_reports_timed_samples():
    """The reference arm times bounded samples of the workload on the host
    cores: its steps' measured time fits in the run's wall time, and its value
    is the sample's share of 2mnk over that time."""
    import json
    import time
    env = dict(os.environ)
    for key in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(key, None)
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", "256", "--steps", "3",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    wall = time.perf_counter() - t0
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 1
    assert (line["steps"] + line["warmup"]) * line["ms_per_step"] / 1e3 <= wall
    P, R = line["config"]["sample_products"], line["config"]["products"]
    assert 1 <= P <= R
    assert abs(line["value"] - 2.0 * 256 ** 3 * P / R / (line["ms_per_step"] / 1e3) / 1e12) <= 1e-9 * line["value"]
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
