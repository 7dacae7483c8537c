"""The benchmark's multi-rank path on CPU: world size 2 over gloo.  Each rank
is an independent replica; the reported time is the maximum over ranks."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
    value = bench.views_per_s(steps=100, world=world, device_ms=ms)
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_two_rank_replicas_take_max_time():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == pytest.approx(2 * 100 / 0.015)
