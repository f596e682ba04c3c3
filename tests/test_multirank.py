"""The N>1 path of bench.py on CPU (gloo, world_size 2).

The C2C path does not exchange data between GPUs: N GPUs run N independent
replicas.  What multi-rank adds is host logic: the barrier, the max over
ranks of the step time, the whole-job aggregate, and rank 0 alone running
and printing the reference arm.  Those are exercised here on CPU ranks.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    dist = bench.dist_init(world, use_cuda=False)
    local_ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
    ms, rate = bench.aggregate(dist, local_ms, units_per_rank=1.0e9)
    dist.barrier()
    q.put((rank, ms, rate))
    dist.destroy_process_group()


def test_aggregate_is_max_over_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(world))
    for rank, ms, rate in res:
        assert ms == pytest.approx(15.0)                 # the slowest rank's time
        assert rate == pytest.approx(2 * 1.0e9 / 15e-3)  # all ranks' units / that time


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    bench.main(["--impl", "reference", "--workload", "1d_4096", "--steps", "1", "--warmup", "0"])
    assert capsys.readouterr().out == ""
    monkeypatch.setenv("RANK", "0")
    bench.main(["--impl", "reference", "--workload", "1d_4096", "--steps", "2", "--warmup", "1"])
    import json
    line = json.loads(capsys.readouterr().out.strip())
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
