"""Partitioning a population of designs across GPUs (one process per GPU).

Designs are independent, so a population shards by design with no data-path
collective: each rank evaluates its own designs and the host gathers three numbers per
design. The work of a design is its ray count (wavelengths x rays per wavelength); the
partition is the longest-processing-time greedy rule (largest design first, to the
least-loaded rank), which is within 4/3 of the optimal makespan and depends only on
the work list, so every rank computes the same partition without communicating.
"""
from __future__ import annotations

from typing import Sequence


def shard_by_work(work: Sequence[float], world: int) -> list[list[int]]:
    """Design indices per rank; each list is in ascending index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-float(work[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(work[i])
    return [sorted(p) for p in parts]


def shard_for_rank(work: Sequence[float], rank: int, world: int) -> list[int]:
    return shard_by_work(work, world)[rank]
