"""The multi-process path of bench.py on CPU: two gloo ranks (the reference arm's backend) run the
barrier and the max-over-ranks timing that bracket the timed region.  The GPU arm uses the same two
helpers over NCCL; its ranks route independent replicas with no collective on the data path."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_init(argparse.Namespace(impl="reference"))
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + rank, w)  # rank r "took" 1 + r seconds
    out.put((rank, t))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_slowest_rank_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(out.get(timeout=5) for _ in procs)
    assert got == [(0, 2.0), (1, 2.0)]
