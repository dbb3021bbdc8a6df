"""The multi-rank path of bench.py on CPU (gloo, world size 2): the systems of each
rank are independent replicas, so the only collective is the max-over-ranks of the
timed seconds, and the reference arm runs on rank 0 alone."""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world,
                            init_method=f"tcp://127.0.0.1:{port}")
    import bench

    q.put((rank, bench.max_over_ranks(1.5 + rank, world, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_reference_arm_silent_on_other_ranks(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, cpu_steps, pad, gpus, workload = 3, 3, 0.2, 2, "shear_n16384_phi086"

    bench.run_reference_arm(Args, {"n": 16384}, rank=1, world=2)
    assert capsys.readouterr().out == ""
