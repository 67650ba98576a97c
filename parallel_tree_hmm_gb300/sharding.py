"""Forests across GPUs: one process per GPU, trees partitioned by node count.

Trees are independent, so a forest shards with no exchange on the data path:
each rank reserves a workspace for its share of the trees and contracts it
alone. The only collective is the optional total log partition (a scalar
sum over ranks). The per-tree work of the sum-product and its adjoint is
proportional to the node count, so ranks are balanced by nodes.
"""
from __future__ import annotations

import heapq
from typing import Sequence

import numpy as np


def partition_trees(node_counts: Sequence[int], world: int) -> list[list[int]]:
    """Greedy longest-processing-time partition of trees over `world` ranks:
    trees by decreasing node count (ties by index), each to the rank with the
    fewest nodes so far (ties by rank). Returns, per rank, its tree indices
    in increasing order. Every tree lands on exactly one rank, and no rank
    holds more than the average load plus the largest tree."""
    if world < 1:
        raise ValueError("world must be at least 1")
    counts = np.asarray(node_counts, dtype=np.int64)
    order = sorted(range(len(counts)), key=lambda t: (-int(counts[t]), t))
    heap = [(0, rank) for rank in range(world)]
    shares: list[list[int]] = [[] for _ in range(world)]
    for tree in order:
        load, rank = heapq.heappop(heap)
        shares[rank].append(tree)
        heapq.heappush(heap, (load + int(counts[tree]), rank))
    return [sorted(share) for share in shares]


def sum_log_partitions(local_log_partitions, dist=None) -> float:
    """Sum over all trees of all ranks of log Z (FP64): this rank's values
    summed, then an all-reduce across the process group when one is given."""
    local = float(np.sum(np.asarray(local_log_partitions, dtype=np.float64)))
    if dist is None:
        return local
    import torch

    on_gpu = dist.get_backend() == "nccl"
    total = torch.tensor([local], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(total, op=dist.ReduceOp.SUM)
    return float(total.item())
