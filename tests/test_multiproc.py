"""The multi-rank host logic of bench.py on CPU: two gloo ranks, each its own
replica, the job time is the max over ranks and the whole-job rate counts every
rank's work ("replicas only": the path has no exchange between GPUs)."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    bench.barrier(ws)
    t = bench.reduce_max(1.0 + rank, ws)      # per-rank "elapsed seconds"
    out[rank] = (ws, r, local, t)
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == (2, 0, 0, 2.0) and res[1] == (2, 1, 1, 2.0)
