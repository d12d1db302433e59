"""Assignment of independent cloths to ranks (one process per GPU).

Cloths of a batch never interact, so a multi-GPU run splits the cloth list
across ranks and steps each share with no collective in the step.  The split
balances the per-step cost, which grows with the vertex count times the
solver iterations (the projection) plus the triangle count (the collision
stages): longest-processing-time first, ties to the lowest rank, so every rank
computes the same assignment from the same list without communicating.
"""
from __future__ import annotations

from typing import Sequence


def cloth_cost(spec) -> float:
    """Relative per-step cost of one cloth."""
    return float(spec.num_vertices * max(int(spec.params.solverIterations), 1) + spec.num_triangles)


def balance(costs: Sequence[float], world: int) -> list[list[int]]:
    """Cloth indices per rank (each list in ascending order)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in out]


def my_share(specs: Sequence, rank: int, world: int) -> list[int]:
    """Indices of the cloths rank `rank` of `world` steps."""
    return balance([cloth_cost(s) for s in specs], world)[rank]
