"""Sharding a batch of independent meshes over GPUs (one process per GPU, no collective).

Meshes are independent representations (the reference steps them as separate tasks of one
FreeMotion pass, FreeMotion.cpp:55-80), so a batch splits across ranks with no data exchange: every
rank computes the same partition from the same mesh list and steps only its own bin.
"""

from __future__ import annotations

import math

import numpy as np


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


# Expected Jacobi-PCG iterations of one implicit-Euler step (CG tolerance 1e-10) of a cube-grid
# mesh: a + b * dt * c / h, with c = sqrt(E / rho) the material's wave speed and h the cube edge
# (the system's condition number grows as (dt c / h)^2). Fitted to the oracle's iteration counts on
# 43 meshes of the 256-mesh batch (E from 1.1e4 to 9.2e5 Pa, 512 to 42,875 nodes): largest error
# 16%, median 2%.
ITER_A = 9.0
ITER_B = 69.0
# Element update, assembly and right-hand side of a step, per node, in units of one CG iteration
# per node (measured on the 256-mesh batch: ~5.4 ms of element-side kernels against ~41 ms of
# solve at ~150 node-weighted iterations).
ELEMENT_ITERS = 20.0


def expected_cg_iterations(mesh, dt: float = 1e-3) -> float:
    """Expected CG iterations of one step of `mesh` (mean E and rho over its elements)."""
    young = float(np.mean(mesh.young))
    rho = float(np.mean(mesh.density))
    return ITER_A + ITER_B * dt * math.sqrt(young / rho) / float(mesh.h)


def mesh_weight(mesh, dt: float = 1e-3) -> float:
    """Work per step of a mesh: its nodes (the system's rows; the non-zeros per row are nearly the
    same for every cube-grid mesh) times the expected CG iterations plus the element-side work.
    A batch waits for its slowest rank, and a mesh's solve time scales with its iterations, which
    vary ~6x with E over the batch's two decades."""
    return float(mesh.num_nodes) * (expected_cg_iterations(mesh, dt) + ELEMENT_ITERS)
