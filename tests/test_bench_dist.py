"""The multi-rank path of bench.py on CPU: two gloo ranks (one process each, 127.0.0.1 rendezvous).

Queries shard trivially, so N ranks run N independent replicas and the only cross-rank step is the timing
reduction (max over ranks).  The reference arm runs on rank 0 alone; the other ranks exit without work."""

import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    v = bench.reduce_max(float(10 * (rank + 1)), torch.device("cpu"))
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, v))


def test_timing_reduction_takes_the_max_over_two_gloo_ranks():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}


def test_reduce_max_without_process_group():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, "cpu") == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_workload_scale_defaults(monkeypatch):
    # every workload runs its chosen form at full size; the parametric workload times its plain FP64 integrator and
    # ablations on a 4% seeded sample of the queries (the plain form on all 1e6 takes about 100 s per step) and
    # trains its network on 1e7 labels; explicit flags win
    sys.path.insert(0, ROOT)
    import bench
    for argv, scale, plain, labels in ((["bench.py"], 1.0, 0.04, 1e7), (["bench.py", "--config", "param"], 1.0, 0.04, 1e7),
                                       (["bench.py", "--config", "robust"], 1.0, 0.04, 1e7),
                                       (["bench.py", "--config", "param", "--scale", "0.1", "--plain-scale", "0.5",
                                         "--labels", "2e6"], 0.1, 0.5, 2e6)):
        monkeypatch.setattr(sys, "argv", argv)
        a = bench.parse()
        assert (a.scale, a.plain_scale, a.labels) == (scale, plain, labels), argv
