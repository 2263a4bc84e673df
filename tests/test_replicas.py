"""Replica logic of bench.py on CPU: two gloo ranks agree on the slowest rank's time and on the whole-job rate, and
the reference arm does its work on rank 0 only."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + rank  # rank 1 is the slow one
        t = bench.max_over_ranks(seconds, dist)
        rate = bench.whole_job_rate(1000.0, t, world)
        out.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [2.0, 2.0]
    assert [r[2] for r in res] == [1000.0, 1000.0]  # 2 ranks x 1000 units / 2 s


def test_max_over_ranks_without_a_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10.0, 2.0, 1) == 5.0


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        steps, warmup, cpu_seconds, workload = 1, 0, 0.1, "cartpole"

    bench.run_reference(Args, ws=2, rank=1)
    assert capsys.readouterr().out == ""


@pytest.mark.parametrize("workload,per_iter", [("cartpole_rmppi", 2 * 2048 * 100 + 9 * 64 * 100),
                                               ("cartpole_tube", 2 * 2048 * 100)])
def test_reference_arm_of_the_host_iterated_controllers(capsys, workload, per_iter):
    """The R-MPPI and Tube-MPPI workloads' reference arm: one line on rank 0 with the workload's config, its sample
    steps per iteration and a CPU sample of the oracle's iteration."""
    import json

    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        steps, warmup, cpu_seconds, instances, precision = 1, 0, 0.1, 256, None

    Args.workload = workload
    bench.run_reference(Args, ws=1, rank=0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"].startswith(workload) and line["config"]["sample_steps_per_iter"] == per_iter
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
