"""Multi-rank aggregation of bench.py (replicas only) on CPU with gloo,
world size 2: the timed duration is the max over ranks and the throughput
counts both ranks' bytes."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ffcz_gb300 import replicas

    assert replicas.world() == (rank, world)
    replicas.barrier()
    secs = [0.5, 2.0][rank]
    rate, t = replicas.throughput(1e9, secs)
    out[rank] = (rate, t)
    dist.destroy_process_group()


def test_two_rank_aggregation():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for r in (0, 1):
        rate, t = out[r]
        assert t == 2.0
        assert rate == pytest.approx(2 * 1e9 / 2.0)
