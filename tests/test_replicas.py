"""Replicas across processes (the only multi-GPU form: one reconstruction
does not shard): every rank reconstructs its own mock (base seed + rank) and
the job's throughput is ranks x steps over the slowest rank's time.  The
host logic of bench.py's torchrun path, on two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, times, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms, value = bench.replica_throughput(times[rank], ws, dist, device="cpu")
        out.put((rank, bench.replica_seed(2024, rank), ms, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    import torch.multiprocessing as mp
    ws, port = 2, _free_port()
    times = [3.0, 4.0]   # ms per step on each rank
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, times, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    seeds = [r[1] for r in res]
    assert seeds == [2024, 2025]                      # every rank its own mock
    for _, _, ms, value in res:
        assert ms == pytest.approx(4.0)                # the slowest rank's step time
        assert value == pytest.approx(2 * 1000.0 / 4.0)   # both ranks' reconstructions per second


def test_one_process_is_its_own_job():
    import bench
    ms, value = bench.replica_throughput(3.5, 1)
    assert ms == 3.5 and value == pytest.approx(1000.0 / 3.5)
