"""Sharding of the batched form across processes (one GPU per process).

Molecules are independent: no data exchange happens during their SCC cycles, so each rank solves its
own share with no collective on the data path. Shares are balanced by the cost model of one SCC
iteration, n^3 per molecule (the dense eigensolve dominates), with the greedy longest-first rule
(each molecule in decreasing cost goes to the currently lightest rank). Results are gathered on the
host afterwards (``gather_to_root``).
"""
from __future__ import annotations

import heapq
from typing import List, Sequence


def shard_by_cost(n_orbitals: Sequence[int], world: int) -> List[List[int]]:
    """Molecule indices per rank; every molecule exactly once, each list in increasing order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(n_orbitals)), key=lambda i: (-int(n_orbitals[i]) ** 3, i))
    heap = [(0, r) for r in range(world)]
    shares: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + int(n_orbitals[i]) ** 3, r))
    return [sorted(s) for s in shares]


def share_cost(n_orbitals: Sequence[int], share: Sequence[int]) -> int:
    return sum(int(n_orbitals[i]) ** 3 for i in share)


def gather_to_root(local: dict, share: Sequence[int], n_total: int):
    """Per-molecule results of this rank ({key: list aligned with share}) gathered on rank 0 into
    lists of length n_total in global molecule order (other ranks get None). Uses the default
    torch.distributed process group (any backend that supports object collectives)."""
    import torch.distributed as dist
    world = dist.get_world_size()
    payload = (list(share), local)
    gathered = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(payload, gathered, dst=0)
    if dist.get_rank() != 0:
        return None
    out = {}
    for idx, res in gathered:
        for key, vals in res.items():
            col = out.setdefault(key, [None] * n_total)
            for i, v in zip(idx, vals):
                col[i] = v
    return out
