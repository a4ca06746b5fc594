"""Replica aggregation of bench.py over torch.distributed (gloo, CPU).

The path has no intra-member exchange, so N GPUs run N independent
replicas; the whole-job value is every rank's points over the slowest
rank's time.  Two CPU ranks check that reduction.
"""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 if rank == 0 else 250.0  # rank 1 is the slow replica
    value, ms_all = bench.replica_value(dist, 1.0e9, ms, device="cpu")
    out[rank] = (value, ms_all)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_value_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for r in (0, 1):
        value, ms_all = out[r]
        assert ms_all == 250.0
        assert value == pytest.approx(2 * 1.0e9 / 0.25)
