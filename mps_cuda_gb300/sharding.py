"""Multi-GPU partitioning of independent scenes (host logic).

The DFSPH step of one scene does not shard without a halo exchange, so N GPUs run replicas
(independent scenes or seeds).  Batched runs split their scenes over ranks with a greedy
largest-first bin packing on particle counts; no collective touches the data path, only the
per-rank statistics are gathered at the end.
"""
from __future__ import annotations


def partition_scenes(counts: list[int], world: int) -> list[list[int]]:
    """Assigns scene indices to `world` ranks, balancing total particles (deterministic)."""
    if world <= 0:
        raise ValueError("world must be positive")
    order = sorted(range(len(counts)), key=lambda i: (-counts[i], i))
    loads = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += counts[i]
    return [sorted(p) for p in parts]


def imbalance(counts: list[int], parts: list[list[int]]) -> float:
    loads = [sum(counts[i] for i in p) for p in parts]
    mean = sum(loads) / max(1, len(loads))
    return max(loads) / mean if mean > 0 else 1.0
