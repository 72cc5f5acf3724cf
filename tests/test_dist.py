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


def _shard_rank_main(rank, world, port, q):
    """One rank of the sharded batch: partition the batch by work, transform
    this rank's share with the CPU oracle (standing in for the rank's GPU), and
    gather every rank's results on rank 0 over gloo."""
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist
    import oracle as O
    from numrs_gb300 import shard
    from numrs_gb300 import workloads as W
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes, u = W.batch_c3(count=600, kmin=6, kmax=12)
    host = W.batch_c3_data(sizes, u)
    parts = shard.partition_by_work(sizes, world)
    mine = parts[rank]
    arrs = [host[i].copy() for i in mine]
    O.fft_batch(arrs, 1)
    gathered = [None] * world
    dist.all_gather_object(gathered, (rank, parts, mine, arrs))
    if rank == 0:
        q.put(gathered)
    dist.destroy_process_group()


def test_gloo_two_ranks_batch_partition():
    """The batch splits across two ranks with no data-path collective: both
    ranks compute the same partition, every transform lands on exactly one
    rank, the work is balanced, and the gathered results equal the oracle's
    unpartitioned batch."""
    pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp
    import oracle as O
    from numrs_gb300 import shard
    from numrs_gb300 import workloads as W
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sizes, u = W.batch_c3(count=600, kmin=6, kmax=12)
    host = W.batch_c3_data(sizes, u)
    parts0 = gathered[0][1]
    assert all(g[1] == parts0 for g in gathered)
    owner = {}
    for rank, _, mine, _ in gathered:
        for i in mine:
            assert i not in owner
            owner[i] = rank
    assert sorted(owner) == list(range(len(sizes)))
    work = [sum(shard.transform_work(sizes[i]) for i in g[2]) for g in gathered]
    assert max(work) / min(work) < 1.01
    refs = [a.copy() for a in host]
    O.fft_batch(refs, 1)
    for rank, _, mine, arrs in gathered:
        for i, a in zip(mine, arrs):
            assert np.array_equal(a, refs[i])


def test_partition_by_work_edge_cases():
    from numrs_gb300 import shard
    assert shard.partition_by_work([], 3) == [[], [], []]
    assert shard.partition_by_work([64], 2) == [[0], []]
    parts = shard.partition_by_work([1 << 14] * 4 + [64] * 8, 4)
    assert sorted(i for p in parts for i in p) == list(range(12))
    # the four large transforms go one to each rank, the small ones two each
    assert [sum(1 for i in p if i < 4) for p in parts] == [1, 1, 1, 1]
    assert [len(p) for p in parts] == [3, 3, 3, 3]
    with pytest.raises(ValueError):
        shard.partition_by_work([8], 0)
