"""bench.py at N > 1 runs N independent replicas (the path does not shard in
this build): the whole-job value is the cells of all ranks over the slowest
rank's time.  Checked with two gloo ranks on the CPU."""
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
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [100.0, 250.0][rank]
    cells = [1000, 3000][rank]
    v, t, n = bench.replica_throughput(ms, cells, dist)
    out[rank] = (v, t, n)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        v, t, n = out[r]
        assert t == 250.0 and n == 4000
        assert v == pytest.approx(4000 / 0.25)


def test_replica_throughput_single():
    import bench

    assert bench.replica_throughput(50.0, 100) == (2000.0, 50.0, 100)
