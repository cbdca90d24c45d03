"""Replica combination for N > 1 (one process per GPU, no data-path collective):
two gloo ranks on CPU with different per-rank work and times."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oofem_gb300 import replicas
    ws, r, lr = replicas.env()
    units = 1000.0 * (rank + 1)          # rank 0: 1000 DOFs, rank 1: 2000 DOFs
    secs = 0.5 + rank                    # rank 0: 0.5 s, rank 1: 1.5 s
    replicas.barrier()
    out[rank] = (ws, r, replicas.max_over_ranks(secs), replicas.sum_over_ranks(units),
                 replicas.job_throughput(units, secs))
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_max_time_and_total_work():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    with mp.get_context("spawn").Manager() as mgr:   # no fork of this (threaded) process
        out = mgr.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ws, r, tmax, total, thr = res[rank]
        assert (ws, r) == (world, rank)
        assert tmax == 1.5
        assert total == 3000.0
        assert thr == pytest.approx(3000.0 / 1.5)


def test_single_process_is_identity():
    from oofem_gb300 import replicas
    assert replicas.max_over_ranks(2.5) == 2.5
    assert replicas.job_throughput(10.0, 2.0) == 5.0
