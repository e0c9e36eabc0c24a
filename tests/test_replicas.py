"""Replicas-only multi-GPU bench logic on CPU: two gloo ranks, the whole-job throughput
uses the slowest rank's time and counts every rank's cells (no data-path exchange)."""

import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.replica_throughput([10.0, 12.5][rank], 1000, 4, world, None)
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_report_max_time_and_summed_cells():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 12.5
        assert value == pytest.approx(2 * 1000 * 4 / 0.0125)


def test_single_rank_needs_no_process_group():
    import bench
    ms, value = bench.replica_throughput(5.0, 100, 2, 1)
    assert ms == 5.0 and value == pytest.approx(100 * 2 / 0.005)
