"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The Align phase has no exchange step: every rank aligns its own replica of
the pair list (weak scaling) and only the step time is reduced across ranks
(maximum).  This runs that logic in two spawned processes over gloo on
127.0.0.1, no GPU involved.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import numpy as np
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, local = bench.dist_setup()
    pairs = np.arange(20, dtype=np.int32).reshape(10, 2)
    mine = bench.shard(pairs, w, r)
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + rank, w)
    out[rank] = (w, r, len(mine), t)
    dist.destroy_process_group()


def test_two_rank_weak_scaling_logic():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    assert sorted(out.keys()) == [0, 1]
    for rank in range(world):
        w, r, n, t = out[rank]
        assert (w, r) == (world, rank)
        assert n == 10          # full replica per rank
        assert t == 2.0         # max over ranks
