"""The replica path of bench.py under torchrun, on CPU: two gloo ranks agree on
the job's time (its slowest rank's) and on the whole-job rate, and the
reference arm runs on rank 0 only (the other ranks return without work)."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = (40.0, 55.0)[rank]
        t = bench.max_over_ranks(ms, dist)
        q.put((rank, t, bench.job_rate(world, 1000, 5, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_job_time_and_rate():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [55.0, 55.0]
    assert all(abs(g[2] - 2 * 1000 * 5 / 0.055) < 1e-6 for g in got)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import types

    import bench
    args = types.SimpleNamespace(workload="fov3c", steps=1, warmup=0)
    assert bench.reference_arm(args, rank=1, world=2) is None
    assert capsys.readouterr().out == ""
