"""Multi-rank host logic of bench.py on CPU: world_size-2 gloo ranks.  The GPU
path runs independent replicas per rank (no data-path collective); the only
cross-rank operations are the barrier and the max-over-ranks time."""
import os
import socket
import sys

import pytest
import torch.distributed as tdist
import torch.multiprocessing as tmp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist()  # gloo: no CUDA in this container
    assert d.world == world and d.rank == rank
    d.barrier()
    local_ms = 10.0 * (rank + 1)
    mx = d.max(local_ms)
    q.put((rank, mx, d.pg.get_backend()))
    d.close()


def test_two_ranks_max_over_ranks():
    world, port = 2, _free_port()
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    assert [r[1] for r in res] == [20.0, 20.0]
    assert all(r[2] == "gloo" for r in res)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(None, 3.5) == 3.5
