"""The multi-GPU path is replicas only: each rank runs its own lattice, with no data-path
collective. The bench's whole-job figure takes the maximum time over ranks and sums the node
updates. Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [40.0, 55.0][rank]
    tmax, value = bench.replica_throughput(ms, 1000, 10, world, dist, "cpu")
    out[rank] = (tmax, value)
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        tmax, value = out[r]
        assert tmax == 55.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.055 / 1e6)


def test_replica_throughput_one_rank():
    import bench
    assert bench.replica_throughput(20.0, 500, 4, 1) == (20.0, pytest.approx(500 * 4 / 0.02 / 1e6))
