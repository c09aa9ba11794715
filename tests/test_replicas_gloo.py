"""The multi-GPU form of the benchmark runs independent replicas (one mesh per
rank, no data-path collective): the step time is the slowest rank's and the
value counts every rank's elements.  Checked with 2 gloo ranks on the CPU."""
import os

import pytest
import torch.multiprocessing as mp


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ms_local = 100.0 if rank == 0 else 250.0          # rank 1 is slower
    ms_step, value = bench.replica_throughput(ms_local, 10, 1000.0, world, dist, "cpu")
    out[rank] = (ms_step, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in (0, 1):
        ms_step, value = out[r]
        assert ms_step == pytest.approx(25.0)                       # max over ranks / steps
        assert value == pytest.approx(2 * 1000.0 / 25e-3 / 1e6)     # both ranks' elements
