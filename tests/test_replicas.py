"""bench.py's multi-process path on the CPU (gloo, world size 2).  The
solve does not shard (replicas only): every rank runs the whole step, the
step time is the slowest rank's, rank 0 alone prints, and the reference
arm's other ranks exit without work."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r measured 10 + r ms: every rank reports the slowest
        q.put((rank, bench.reduce_max_over_ranks(10.0 + rank, "cpu")))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_step_time_is_max_over_ranks_gloo():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert got == [(0, 11.0), (1, 11.0)]
    assert all(p.exitcode == 0 for p in procs)


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(bench.args_parse([])) == 0
    assert capsys.readouterr().out == ""
