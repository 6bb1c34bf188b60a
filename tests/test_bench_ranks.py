"""bench.py with N > 1 processes (replicas: every rank solves its own copy of
the workload, no collective in the data path): the step time is the slowest
rank's (checked with two gloo ranks on the CPU), and the reference arm runs on
rank 0 only (the other ranks return without work or output)."""
import argparse
import io
import os
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.max_over_ranks(1.0 + rank, world, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == {0: 2.0, 1: 2.0}


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(steps=1, warmup=0, gpus=2)
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(args, rank=1, world=2) == 0
    assert buf.getvalue() == ""
    assert bench.max_over_ranks(3.5, 1) == 3.5
