"""The N > 1 path of bench.py on the host: replicas under torch.distributed (gloo,
world size 2, 127.0.0.1) agree on the slowest rank's time, and the reference arm runs on
rank 0 only (the other ranks exit without work)."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _max_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, torch.device("cpu"))
        dist.barrier()
        out.put((rank, ms))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_reference_arm_only_on_rank0(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    args = type("A", (), {"warmup": 0, "steps": 1, "n": 28, "gpus": 2, "seed": 1, "workload": "circuit"})()
    bench.run_reference(args)
    bench.run_reference_contract(args)
    assert capsys.readouterr().out == ""
