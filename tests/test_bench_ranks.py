"""The multi-rank path of bench.py on CPU: two gloo ranks time different
spans, both see the slowest one, and the job value counts every rank's
replica.  Under torchrun the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.rank_barrier(world, dist)
        mine = 1.0 + rank  # rank 1 is the slow one
        worst = bench.slowest_over_ranks(mine, world, dist, device="cpu")
        out.put((rank, worst, bench.job_mlups(world, 1000, 10, worst)))
        bench.rank_barrier(world, dist)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_span():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.0, 2.0]
    # 2 replicas x 1000 nodes x 10 steps in 2 s
    assert all(abs(g[2] - 2 * 1000 * 10 / 2.0 / 1e6) < 1e-15 for g in got)


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_over_ranks(3.5, 1, None) == 3.5
    bench.rank_barrier(1, None)
    assert bench.job_mlups(1, 100, 5, 0.5) == 100 * 5 / 0.5 / 1e6


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
