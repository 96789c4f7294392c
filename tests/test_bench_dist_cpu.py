"""bench.py's replicas path across ranks, on CPU with gloo (world size 2):
whole-job figures are the max of the ranks' times and the sum of their
operations; the reference arm prints from rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dev_s, e2e_s, ops = bench.combine_ranks(dist, 1.0 + rank, 3.0 - rank, 100 * (rank + 1), "cpu")
    dist.barrier()

    class Args:
        gpus, steps, warmup = world, 1, 3
    ref = bench.reference_arm(Args, rank, None) if rank != 0 else "rank0"
    out[rank] = (dev_s, e2e_s, ops, ref)
    dist.destroy_process_group()


def test_combine_ranks_gloo_world_size_2():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        dev_s, e2e_s, ops, _ = out[rank]
        assert dev_s == 2.0 and e2e_s == 3.0 and ops == 300
    assert out[1][3] is None  # non-zero ranks print nothing for the reference arm
