"""The benchmark's N > 1 path on the CPU: world size 2 over gloo.  Replicas of
the workload run on every rank; the job's time is its slowest rank's, and the
whole-job value counts every rank's products.  The reference arm runs on rank
0 only."""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(times[rank], dist, torch.device("cpu"))
    value = bench.job_gbs(2.0e9, world, t)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, value))


def test_two_ranks_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    times = [0.004, 0.005]
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [0.005, 0.005]
    # both ranks' products (2 GB each) over the slower rank's 5 ms
    assert all(abs(g[2] - 800.0) < 1e-9 for g in got)


def test_one_rank_is_its_own_slowest():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, None, None) == 0.25
    assert bench.job_gbs(1.0e9, 1, 0.5) == 2.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
