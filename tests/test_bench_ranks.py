"""bench.py's multi-GPU host logic on CPU: replicas (one process per GPU, no collective on the
data path) reduce their timed-region lengths to the maximum over ranks (gloo here, NCCL on GPUs)
and report the whole job's rate; the reference arm does its CPU work on rank 0 only."""

import os
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT

sys.path.insert(0, ROOT)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = 1000.0 * (rank + 1)  # rank 1 is the slower replica
    total = bench.max_over_ranks(local_ms)
    q.put((rank, total, bench.replica_rate(world, 3, total)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2000.0, 2000.0]
    assert all(abs(o[2] - 3.0) < 1e-12 for o in out)  # 2 replicas x 3 solves in 2 s


def test_single_process_needs_no_group():
    import bench

    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replica_rate(1, 4, 2000.0) == 2.0


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    assert bench.run_reference(bench.parse()) == 0  # returns at once: no oracle work on rank 1
