"""The multi-rank path of bench.py (one replica per rank, barrier, max of
the per-rank times) on two gloo ranks on CPU."""
import os
import socket
import sys
from pathlib import Path

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, str(REPO))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    bench.barrier()
    m = bench.max_over_ranks(10.0 + rank)
    out[rank] = (ws, r, local, m)
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
    port = _free_port()
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == (2, 0, 0, 11.0)
    assert out[1] == (2, 1, 1, 11.0)


def test_single_process_identity():
    sys.path.insert(0, str(REPO))
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
