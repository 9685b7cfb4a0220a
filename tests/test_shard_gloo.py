"""Multi-process path on CPU: two gloo ranks split a ragged batch of
correlations by cost and gather the results; the gathered outputs equal a
single-process computation.  (The GPU kernel is replaced by the oracle here:
this tests the host-side partitioning and gathering.)"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from xcorr import shard


def test_shard_balances_by_cost():
    costs = [100, 1, 1, 1, 50, 50]
    parts = shard.shard(costs, 2)
    loads = [sum(costs[i] for i in p) for p in parts]
    assert sorted(i for p in parts for i in p) == list(range(6))
    assert sorted(loads) == [101, 102]  # 100+1+1 | 50+50+1
    assert shard.shard([5, 5, 5], 1) == [[0, 1, 2]]
    with pytest.raises(ValueError):
        shard.shard([1], 0)


def make_batch(seed=4, n=12):
    rng = np.random.default_rng(seed)
    lefts, rights = [], []
    for _ in range(n):
        hl, wl, hr, wr = rng.integers(3, 17, size=4)
        lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(np.float32))
        rights.append(rng.uniform(-1, 1, (hr, wr)).astype(np.float32))
    return lefts, rights


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lefts, rights = make_batch()
    costs = [shard.pair_cost(l.shape, r.shape) for l, r in zip(lefts, rights)]

    def compute(idx):
        return oracle.run_pairs([lefts[i] for i in idx], [rights[i] for i in idx]) if idx else []

    full = shard.run_sharded(len(lefts), costs, compute, rank, world)
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        q.put([np.asarray(x) for x in full])


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_gather_the_full_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from oracle import oracle
    lefts, rights = make_batch()
    ref = oracle.run_pairs(lefts, rights)
    assert len(full) == len(ref)
    for a, b in zip(full, ref):
        np.testing.assert_array_equal(a, b)
