"""Ensembles over several GPUs: one process per GPU, members partitioned by cost.

Ensemble members (independent SSA/DIVA solves, each on its own mesh) shard with no exchange on
the data path: every rank solves its share of the members side by side on its GPU
(`ensemble_solve`), and the only communication is a host-side gather of the per-member results
at the end.  The partition balances the ranks' work by a cost per member (stored stiffness
blocks, or vertices as a proxy) with the longest-processing-time rule, deterministically, so
every rank computes the same partition without exchanging it.

    idx = shard(rank, world, costs)            # the members this rank solves
    ...solve members idx on this rank's GPU...
    results = gather_results({i: result_i for i in idx})   # every rank: all members' results
"""
from __future__ import annotations

import heapq


def partition_members(costs, world: int):
    """Member indices per rank: members in decreasing cost (ties by index), each to the rank with
    the least total so far (ties by rank).  Lists are returned in increasing member order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(p) for p in parts]


def shard(rank: int, world: int, costs):
    """The member indices `rank` solves."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return partition_members(costs, world)[rank]


def gather_results(local: dict):
    """Merge {member index: result} over all ranks (host-side all-gather of picklable results);
    without an initialised process group the local dict is returned.  Every rank receives the
    merged dict; a member reported by two ranks is an error."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return dict(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, dict(local))
    merged = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError(f"member {k} reported by two ranks")
            merged[k] = v
    return merged


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the slowest rank's time), on `device` (None: CPU
    tensor, for gloo); the value itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
