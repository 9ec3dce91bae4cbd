"""Replicas over several GPUs: independent molecules, no device collective.

The path does not shard inside one molecule (one CCSD solve lives on one
GPU); a batch of independent molecules (or field points) is split into
contiguous shards of nearly equal work, each rank solves its shard on its own
GPU, and rank 0 gathers the scalar results over the host process group
(``torch.distributed`` with gloo, or whatever the caller initialised).
"""
from __future__ import annotations

import numpy as np


def work(mol) -> float:
    """Relative CCSD cost of one molecule: o^3 v^3 (the ring contractions)."""
    n = mol.n_sites
    o = mol.n_electrons // 2
    v = n - o
    return float(o) ** 3 * float(v) ** 3


def shard(molecules, rank: int, world: int):
    """Indices of the molecules rank `rank` solves: contiguous, balanced by work."""
    if world <= 1:
        return list(range(len(molecules)))
    w = np.array([work(m) for m in molecules])
    cum = np.cumsum(w)
    total = cum[-1] if len(cum) else 0.0
    lo, hi = total * rank / world, total * (rank + 1) / world
    mid = cum - w / 2
    return [i for i in range(len(molecules)) if lo <= mid[i] < hi or (rank == world - 1 and mid[i] >= hi)]


def gather(local: dict, rank: int, world: int):
    """Gather {index: result} dicts from every rank onto rank 0 (host collective)."""
    if world <= 1:
        return local
    import torch.distributed as dist
    bucket = [None] * world
    dist.all_gather_object(bucket, local)
    if rank != 0:
        return None
    out = {}
    for b in bucket:
        out.update(b)
    return out
