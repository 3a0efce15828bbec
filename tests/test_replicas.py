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


def test_reference_arm_json_line_small(monkeypatch, capsys):
    """The reference arm on a small mesh, on the CPU: one JSON line with the
    contract's keys, the CPU port as its baseline and no host-device bytes."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    a = bench.args_parse(["--impl", "reference", "--nex", "8", "--ney", "8",
                          "--nez", "4", "--steps", "1", "--warmup", "1",
                          "--cpu-iters", "2"])
    assert bench.run_reference(a) == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "s" and d["value"] > 0 and d["higher_is_better"] is False
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "s",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and d["reference_iterations"] > 0
