"""Multi-GPU layout of this path is replicas only: ranks run independent
solves and only the timing is combined (max over ranks).  This checks the
combination with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    v, t = bench.replica_rate(10, 1.0 + rank, ws, "cpu")
    out[rank] = (v, t)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn", join=True)
    for r in range(ws):
        v, t = out[r]
        assert t == pytest.approx(2.0)
        assert v == pytest.approx(ws * 10 / 2.0)


def test_replica_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(20, 0.5, 1) == (40.0, 0.5)
