"""The N > 1 path of bench.py on CPU (gloo, world size 2).

Each rank renders an independent replica of the workload (the path does not
shard across devices: no collective touches the render), so the only
multi-rank logic is the timing: the slowest rank's time, every rank's work
counted, rank 0 alone reporting and rank 0 alone timing the CPU reference.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    slowest = bench.rank_max(1.0 + rank, dist)
    rate, seconds = bench.job_rate(100.0, 2.0 + 3.0 * rank, world, dist)
    dist.barrier()
    q.put((rank, slowest, rate, seconds))
    dist.destroy_process_group()


def test_two_ranks_time_the_slowest_and_count_every_rank():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate, seconds in out:
        assert slowest == 2.0       # max over ranks of 1 + rank
        assert seconds == 5.0       # the slower rank's 2 + 3
        assert rate == 100.0 * 2 / 5.0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_max(3.5) == 3.5
    assert bench.job_rate(10.0, 2.0, 1) == (5.0, 2.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit 0 at once, printing
    nothing and loading nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
