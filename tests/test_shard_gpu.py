"""The sharded path on the GPU: two processes (gloo for the gather) each run
their cost-balanced share of a ragged batch through the library's ragged plan
on the visible GPU; the gathered outputs must match the oracle.  The ranks'
kernels are independent (no rank waits on another's kernel); only the host
gather joins them."""
import os
import socket

import numpy as np
import pytest

from helpers import rel_to_max

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def make_batch(seed=9, n=10):
    rng = np.random.default_rng(seed)
    lefts, rights = [], []
    for _ in range(n):
        hl, wl, hr, wr = rng.integers(8, 120, size=4)
        lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(np.float32))
        rights.append(rng.uniform(-1, 1, (hr, wr)).astype(np.float32))
    return lefts, rights


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from xcorr import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lefts, rights = make_batch()
    full = shard.correlate_pairs_sharded(lefts, rights, rank, world)
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


def test_two_ranks_share_a_ragged_batch_on_the_gpu():
    import torch.multiprocessing as mp

    from oracle import oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    lefts, rights = make_batch()
    refs = oracle.run_pairs(lefts, rights, threads=8)
    assert len(full) == len(refs)
    for k, (o, r) in enumerate(zip(full, refs)):
        assert o.shape == r.shape, k
        assert rel_to_max(o, r) <= 1e-5, k
