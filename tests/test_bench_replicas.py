"""CPU tests of the replicas path of bench.py (N > 1 ranks, one GPU each):
the only collective is the maximum of the timed values over the ranks, run
here as two gloo processes; the reference arm runs on rank 0 alone."""

import os
import socket
import sys
import types
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    q.put((rank, bench.max_over_ranks([10.0 + rank, 5.0 - rank, 7.5], 2)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, [11.0, 5.0, 7.5]), (1, [11.0, 5.0, 7.5])]


def test_max_over_ranks_one_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([3, 4.5], 1) == [3.0, 4.5]


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    args = types.SimpleNamespace(workload="photo1024_default", steps=1, warmup=0, cpu_budget=0.1)
    assert bench.run_reference(args, 1, 2) is None
    assert capsys.readouterr().out == ""
