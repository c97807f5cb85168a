"""Multi-GPU form: independent replicas (one engine per rank, no data-path
collective), the path SIFT shards along (whole images). The host side of it —
rank discovery, the barrier and the max-over-ranks timing reduction bench.py
uses — runs here as two gloo ranks on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, local = bench.dist_setup()
    bench.barrier(w)
    # each rank "timed" its own replica; the job time is the slowest rank's
    t = bench.allreduce_max(w, 1.0 + rank)
    value = w * 10 / t  # images of all ranks / max rank time
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, local, w, t, value))


def test_two_rank_replicas_reduce_max():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[2] == 2 for o in out)
    assert all(o[3] == 2.0 for o in out)      # max over ranks
    assert all(o[4] == 10.0 for o in out)     # 2 ranks x 10 images / 2.0 s


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """--impl reference under torchrun: ranks other than 0 exit without work."""
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload = "512"
        warmup = 0
        steps = 1
        gpus = 2
    assert bench.run_reference(A(), 2, 1) is None
    assert capsys.readouterr().out == ""
