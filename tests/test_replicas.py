"""Multi-GPU runs are replicas only (the step does not shard on one GPU):
every rank runs the case on its own GPU, the job time is the max over
ranks.  The host logic of that (barrier, max over ranks) is exercised here
with world_size 2 on the gloo backend, on CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    bench.barrier(ws)
    out[rank] = bench.max_over_ranks(1.5 + rank, ws)
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ws = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}
