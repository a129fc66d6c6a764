"""The bench's multi-GPU form is replicas only: N independent replicas of the evaluation, the
timed region bracketed by barriers and the time taken as the maximum over ranks.  These
tests run that host logic as two gloo ranks on the CPU (no GPU, no NCCL)."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = 10.0 + 5.0 * rank  # rank 1 is the slower replica
        dist.barrier()
        ms = bench.max_over_ranks(torch, ms_local, dist, "cpu")
        out[rank] = (ms, bench.replica_throughput(world, 40, ms))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(rank_main, args=(world, free_port(), out), nprocs=world, join=True)
        got = dict(out)
    # both ranks see the maximum over ranks; the value counts both replicas' evaluations
    assert got[0][0] == got[1][0] == 15.0
    assert got[0][1] == got[1][1] == pytest.approx(2 * 1e3 * 40 / 15.0)


def test_single_process_needs_no_process_group():
    assert bench.max_over_ranks(torch, 12.5, None, "cpu") == 12.5
    assert bench.replica_throughput(1, 10, 20.0) == pytest.approx(500.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun only rank 0 runs and prints the reference arm; other ranks exit 0."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
