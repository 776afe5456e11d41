"""Multi-GPU runs of bench.py are independent replicas (the path has no
exchange step): the host logic is the max-over-ranks timing and the
whole-job throughput.  Checked here with two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    slowest = bench.replica_max(10.0 + 5.0 * rank, dist)
    q.put((rank, slowest, bench.replicas_throughput(1_000_000, world, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # rank 1 took 15 ms: both ranks report it, and the job built 2 x 1M points in 15 ms
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == pytest.approx(2_000_000 / 15e-3 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=1, warmup=3)
    assert bench.run_reference_arm(args) == 0   # returns at once: no cloud, no oracle run


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_max(12.5, None) == 12.5
