"""The multi-GPU form is replicas only: every rank runs the whole pipeline on its own volume,
with no exchange step. Its host logic - slowest-rank timing and whole-job throughput - is
checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
        ms_max = bench.replica_max(local_ms, world, torch.device("cpu"))
        value = bench.replica_throughput(1000, 3, world, ms_max / 1e3)
        out[rank] = (ms_max, value)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_summed_work():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms_max, value = res[0]
    assert ms_max == 200.0
    assert value == pytest.approx(2 * 1000 * 3 / 0.2 / 1e9)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.replica_max(5.0, 1, None) == 5.0
    assert bench.replica_throughput(10, 2, 1, 4.0) == pytest.approx(5e-9)
