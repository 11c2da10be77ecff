"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): each rank
reconstructs its own realisation and the job time is the max over ranks.
The path itself has no collective (replicas only)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as tdist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seed = bench.replica_seed(1000, rank)
    t = bench.max_over_ranks(10.0 + 5.0 * rank)
    out[rank] = (seed, t)
    tdist.destroy_process_group()


def test_replicas_two_ranks():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    seeds = {out[r][0] for r in range(world)}
    assert len(seeds) == world
    assert all(out[r][1] == 15.0 for r in range(world))
