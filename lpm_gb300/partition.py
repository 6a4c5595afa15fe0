"""Sharding of the direct sum across ranks.

Every target's sum is independent, so a problem shards by target rows with
the sources replicated: rank r evaluates a contiguous, balanced slice of the
targets, and after each evaluation the ranks all-gather the slices (the only
exchange; per RK stage the updated source positions would be all-gathered
the same way).  Ensembles shard by problem with no exchange at all.  In this
environment every box has one GPU, so the GPU benchmark runs replicas; the
partition logic is exercised by multi-process CPU tests (gloo).
"""
from __future__ import annotations


def target_slice(n: int, world: int, rank: int) -> slice:
    """Balanced contiguous slice of n targets for rank (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return slice(start, stop)


def problem_assignment(costs, world: int) -> list[list[int]]:
    """Greedy longest-first assignment of independent problems (ensemble
    members) to ranks by cost, e.g. interactions per evaluation."""
    order = sorted(range(len(costs)), key=lambda i: -costs[i])
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: load[k])
        out[r].append(i)
        load[r] += costs[i]
    return out
