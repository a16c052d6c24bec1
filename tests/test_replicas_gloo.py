"""Multi-GPU path of the benchmark (replicas, one per rank) on CPU with gloo,
world size 2: the slowest rank's time sets the whole-job rate."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = 10.0 + 5.0 * rank          # rank 1 is the slow replica
        ms = bench.max_over_ranks(ms_local, dist, torch.device("cpu"))
        rate = bench.whole_job_rate(1000, ms, world)
        dist.barrier()
        out.put((rank, ms, rate))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in res:
        assert ms == pytest.approx(15.0)
        assert rate == pytest.approx(2 * 1000 / 0.015)
