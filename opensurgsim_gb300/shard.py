"""Sharding a batch of independent meshes over GPUs (one process per GPU, no collective).

Meshes are independent representations (the reference steps them as separate tasks of one
FreeMotion pass, FreeMotion.cpp:55-80), so a batch splits across ranks with no data exchange: every
rank computes the same partition from the same mesh list and steps only its own bin.
"""

from __future__ import annotations


def partition(weights, k: int) -> list:
    """Greedy longest-processing-time bin packing: meshes in decreasing weight (ties by index) go to
    the currently lightest bin (ties by bin index). Deterministic; every index lands in exactly one
    bin; each bin's indices are returned in increasing order. The heaviest bin exceeds the mean load
    by at most the heaviest single weight."""
    if k < 1:
        raise ValueError("k must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    loads = [0.0] * k
    bins = [[] for _ in range(k)]
    for i in order:
        b = min(range(k), key=lambda j: (loads[j], j))
        bins[b].append(i)
        loads[b] += float(weights[i])
    return [sorted(b) for b in bins]


def mesh_weight(mesh) -> float:
    """Work per step of a mesh, proportional to its tets (element pass) and nodes (solve)."""
    return float(mesh.num_tets) + 4.0 * float(mesh.num_nodes)
