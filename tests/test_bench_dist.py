"""The bench's N > 1 path on the CPU: two gloo ranks, the timed region is the
max over ranks and dist_env reads the launcher's environment (the replicas run
no data-path collective)."""

import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, REPO)
    import bench
    ws, r, local = bench.dist_env()
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.job_time_ms(10.0 + 5.0 * rank, ws)
    dist.barrier()
    out[rank] = (ws, r, local, ms)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == (2, 0, 0, 15.0)
    assert res[1] == (2, 1, 1, 15.0)


def test_single_rank_keeps_its_time():
    sys.path.insert(0, REPO)
    import bench
    assert bench.job_time_ms(12.5, 1) == 12.5
