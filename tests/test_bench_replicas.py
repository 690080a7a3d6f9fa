"""CPU test of the replica aggregation bench.py uses under torchrun (gloo, 2 ranks)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.dist_init(world, use_cuda=False)
    # rank r "solves" 8 units in (1 + r) seconds: whole-job rate = 16 / 2
    rate, t = bench.replica_aggregate(d, 1.0 + rank, 8.0, device="cpu")
    out[rank] = (rate, t)
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == pytest.approx((8.0, 2.0))
    assert out[1] == pytest.approx((8.0, 2.0))
