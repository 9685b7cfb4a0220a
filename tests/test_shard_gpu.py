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


def make_batch(seed=9, n=10, big=False):
    """n pairs with sides in 8..119; with `big`, three more of 4e8 to 6e8
    multiply-adds (above the split-BF16 routes' 2^26 and 2^28 thresholds)."""
    rng = np.random.default_rng(seed)
    lefts, rights = [], []
    for _ in range(n):
        hl, wl, hr, wr = rng.integers(8, 120, size=4)
        lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(np.float32))
        rights.append(rng.uniform(-1, 1, (hr, wr)).astype(np.float32))
    if big:
        for hl, wl, hr, wr in [(150, 140, 130, 160), (170, 150, 140, 150), (160, 160, 160, 130)]:
            lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(np.float32))
            rights.append(rng.uniform(-1, 1, (hr, wr)).astype(np.float32))
    return lefts, rights


def _worker(rank, world, port, q, variant=None):
    import torch.distributed as dist

    from xcorr import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lefts, rights = make_batch(big=variant is not None)
    full = shard.correlate_pairs_sharded(lefts, rights, rank, world, variant=variant)
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


@pytest.mark.parametrize("variant", [None, 8])
def test_two_ranks_share_a_ragged_batch_on_the_gpu(variant):
    """variant 8: tile shape 0, the pairs of at least 2^26 multiply-adds on the
    split-BF16 path."""
    import torch.multiprocessing as mp

    from oracle import oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, variant)) for r in range(2)]
    for p in procs:
        p.start()
    full = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    lefts, rights = make_batch(big=variant is not None)
    refs = oracle.run_pairs(lefts, rights, threads=8)
    assert len(full) == len(refs)
    for k, (o, r) in enumerate(zip(full, refs)):
        assert o.shape == r.shape, k
        assert rel_to_max(o, r) <= 1e-5, k
