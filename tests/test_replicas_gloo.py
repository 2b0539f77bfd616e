"""bench.py's replica plumbing (rendezvous, barrier, max over ranks) on CPU, world size 2, gloo."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import bench

    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(10.0 + rank, w)
    out[rank] = t
    import torch.distributed as dist

    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_replicas_take_the_max_over_ranks():
    if torch.cuda.is_available():
        pytest.skip("the gloo replica test runs on CPU-only hosts")
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    assert out[0] == out[1] == 11.0
