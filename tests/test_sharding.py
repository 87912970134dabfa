"""Row-strip sharding of one coupling problem across ranks (the multi-GPU
layout), exercised with world_size-2 gloo process groups on the CPU.

Pairs (l1 <= l2) are independent, so ranks take disjoint l1 rows of balanced
work, compute their rows (here with the oracle) and the host gathers them;
there is no collective on the data path, only the final gather.
"""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, L, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "powerspectra.jl_gb300"))
    from oracle import oracle as o
    from powerspectra_gpu.sharding import row_shards
    rows = row_shards(0, L, world)[rank]
    W = np.linspace(1.0, 2.0, 2 * L + 1)
    M = o.inner_mcm(0, W, 0, L, rows=rows, nthreads=1)
    obj = [None] * world
    dist.all_gather_object(obj, (rows, M))
    if rank == 0:
        full = np.zeros((L + 1, L + 1), order="F")
        seen = np.zeros(L + 1, dtype=int)
        for r, m in obj:
            for l1 in r:
                seen[l1] += 1
                full[l1, l1:] = m[l1, l1:]
                full[l1:, l1] = m[l1:, l1]
        out_q.put((seen.tolist(), full))
    dist.barrier()
    dist.destroy_process_group()


def test_row_shards_balanced():
    from powerspectra_gpu.sharding import row_shards, row_cost
    L = 3071
    for world in (1, 2, 4, 8):
        shards = row_shards(0, L, world)
        allrows = sorted(r for s in shards for r in s)
        assert allrows == list(range(L + 1))
        costs = [sum(row_cost(r, L) for r in s) for s in shards]
        assert max(costs) / min(costs) < 1.01


@pytest.mark.timeout(120)
def test_gloo_two_ranks_gather_equals_single():
    from oracle import oracle as o
    L = 40
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, L, q)) for r in range(2)]
    for p in procs:
        p.start()
    seen, full = q.get(timeout=100)
    for p in procs:
        p.join(30)
        assert p.exitcode == 0
    assert seen == [1] * (L + 1)
    W = np.linspace(1.0, 2.0, 2 * L + 1)
    np.testing.assert_array_equal(full, o.inner_mcm(0, W, 0, L, nthreads=1))
