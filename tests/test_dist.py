"""CPU test of the multi-rank bench plumbing with the gloo backend (world size
2): the barrier and the max-over-ranks timing reduction that bench.py uses when
torchrun launches one rank per GPU.  The ranks here run no GPU work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, loc = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(float(10 * (r + 1)), w)
    q.put((r, w, loc, m))
    dist.destroy_process_group()


def test_gloo_two_ranks_barrier_and_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 0, 20.0), (1, 2, 1, 20.0)]
