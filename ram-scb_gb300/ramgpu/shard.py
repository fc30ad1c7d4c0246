"""Ensemble members across GPUs (one process per GPU).

RAM's species loop has no coupling between species (src/ModRamRun.f90:64-185),
and ensemble members share nothing but the field tables, so a batched
ensemble partitions by member with no exchange in the step: every rank runs
its own members to the end of their runs and the diagnostics are gathered on
rank 0 afterwards.  Members differ in cost (1-4 species, 360-1440 steps), so
the partition balances their work, not their count.
"""
from __future__ import annotations

import heapq


def member_work(species, lengths):
    """Cell-update weight of each member: species count x run length."""
    return [len(s) * int(n) for s, n in zip(species, lengths)]


def partition_members(work, world: int):
    """Members split over `world` ranks by longest-processing-time greedy:
    heaviest member first, each to the rank with the least work so far
    (ties to the lowest rank).  Returns one ascending member list per rank;
    every member appears exactly once.  The heaviest rank carries at most
    4/3 of the optimum (Graham's bound)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda m: (-work[m], m))
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for m in order:
        load, r = heapq.heappop(heap)
        parts[r].append(m)
        heapq.heappush(heap, (load + work[m], r))
    return [sorted(p) for p in parts]


def gather_member_rows(rows: dict, world: int, rank: int, n_members: int, dist=None):
    """Per-member diagnostic rows computed by each rank ({member: row})
    gathered on every rank into one list indexed by member (None for a
    member no rank reported).  dist: torch.distributed (None for world 1)."""
    if world == 1 or dist is None:
        merged = dict(rows)
    else:
        bucket = [None] * world
        dist.all_gather_object(bucket, rows)
        merged = {}
        for part in bucket:
            for m, row in part.items():
                if m in merged:
                    raise RuntimeError(f"member {m} reported by two ranks")
                merged[m] = row
    return [merged.get(m) for m in range(n_members)]
