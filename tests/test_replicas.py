"""The multi-GPU path is replicas only: each rank samples its own walker sets and the
benchmark combines the ranks' figures on the host.  This runs that combination with two
gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    tot = np.array([100.0 + rank, 10.0 * (rank + 1), 1.0])
    tmax = np.array([1.0 + rank, 2.0 - rank, 0.5])
    t, m = bench.combine_ranks(tot, tmax, "cpu")
    out[rank] = (t.tolist(), m.tolist(), bench.replica_seeds(rank))
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_samples_and_take_the_slowest_time():
    world = 2
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        t, m, seeds = out[r]
        assert t == [201.0, 30.0, 2.0]
        assert m == [2.0, 2.0, 0.5]
    assert set(out[0][2]).isdisjoint(out[1][2])
