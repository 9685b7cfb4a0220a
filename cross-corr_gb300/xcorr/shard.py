"""Splitting a batch of correlations over several GPUs (one process each).

Every output matrix of a batch is independent, so a multi-GPU run needs no
data-path collective: each rank computes a share of the outputs from the full
(replicated) inputs, and the shares are gathered once at the end.  Shares are
balanced by multiply-accumulate count (longest-processing-time greedy), which
matters for ragged batches whose pairs differ in size.
"""
from __future__ import annotations

import heapq
from typing import Callable, List, Sequence, Tuple


def pair_cost(left_shape: Tuple[int, int], right_shape: Tuple[int, int]) -> int:
    """Multiply-accumulates of one full correlation: every left element meets
    every right element once."""
    return left_shape[0] * left_shape[1] * right_shape[0] * right_shape[1]


def shard(costs: Sequence[int], world_size: int) -> List[List[int]]:
    """Partition output indices over ranks, heaviest first onto the least
    loaded rank; each rank's list is returned in ascending output order."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0, r) for r in range(world_size)]
    parts: List[List[int]] = [[] for _ in range(world_size)]
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(p) for p in parts]


def run_sharded(n_outputs: int, costs: Sequence[int], compute: Callable[[List[int]], list], rank: int,
                world_size: int, group=None) -> list:
    """Compute this rank's outputs with `compute(indices) -> list of arrays`
    and gather every rank's results into the full, ordered list (on all ranks).
    Uses torch.distributed.all_gather_object, so any backend works (gloo here)."""
    import torch.distributed as dist

    parts = shard(costs, world_size)
    mine = parts[rank]
    results = compute(mine)
    gathered = [None] * world_size
    dist.all_gather_object(gathered, (mine, results), group=group)
    full = [None] * n_outputs
    for idx, res in gathered:
        for i, r in zip(idx, res):
            full[i] = r
    return full


def correlate_pairs_sharded(lefts, rights, rank: int, world_size: int, group=None, dtype: str = "f32",
                            variant=None) -> list:
    """Correlations of the pairs (lefts[i], rights[i]) split over the ranks of
    a process group: each rank runs its cost-balanced share as one ragged
    plan (xcorr.RaggedPlan: one CUDA graph) on its current CUDA device, and
    every rank returns the full, ordered list of output arrays.  `variant`
    picks the plan's variant: None keeps its default (every pair on the plain
    kernel), "auto" autotunes it on the rank's share, an int selects it (for
    FP32, the variants that route the largest pairs through the split-BF16
    path)."""
    import torch

    from . import RaggedPlan

    costs = [pair_cost(l.shape, r.shape) for l, r in zip(lefts, rights)]

    def compute(idx):
        if not idx:
            return []
        plan = RaggedPlan([lefts[i] for i in idx], [rights[i] for i in idx], [(k, k) for k in range(len(idx))],
                          dtype)
        try:
            if variant == "auto":
                plan.autotune()
            elif variant is not None:
                plan.select(int(variant))
            plan.execute()
            torch.cuda.synchronize()
            return plan.outputs()
        finally:
            plan.close()

    return run_sharded(len(lefts), costs, compute, rank, world_size, group)
