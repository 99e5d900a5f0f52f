"""The multi-GPU form of the bench is replicas only (the path fixes one GPU; its
pixels and samples would shard with no exchange but a film sum): every rank
renders the same workload, the job's time is the slowest rank's and its rate
counts every rank's samples. The reduction is checked here with two gloo ranks
on the CPU, through the same helpers bench.py uses."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")  # rank 1 is the slow one
        out.put((rank, slowest, bench.whole_job_rate(1_000_000, world, slowest / 1e3)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_all_samples():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(out.get(timeout=10) for _ in procs)
    assert [r[1] for r in res] == [15.0, 15.0]          # max over ranks on both
    assert res[0][2] == pytest.approx(2 * 1e6 / 0.015 / 1e6)  # both ranks' samples over the slowest time


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(67_108_864, 1, 0.0437) == pytest.approx(67.108864 / 0.0437)
