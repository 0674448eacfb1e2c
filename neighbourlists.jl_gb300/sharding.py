"""Host-side work partitioning for runs with one process per GPU.

A single system is not split (it would need a halo exchange), so several
GPUs run replicas.  Batches of independent systems are split by predicted
pair-buffer bytes with no collective on the data path: each rank builds the
lists of its own systems, and only timings are reduced (max over ranks).
"""
from __future__ import annotations

import heapq
import math
from typing import List, Sequence

import numpy as np

BYTES_PER_PAIR = 44  # i 4 + j 4 + S 12 + R 24 (Int32 indices)


def predicted_pairs(nat: int, cell, cutoff: float, pbc=(True, True, True)) -> float:
    """Expected number of ordered pairs of a homogeneous system:
    nat * rho * 4/3 pi rc^3 (an upper estimate for open boundaries)."""
    vol = abs(float(np.linalg.det(np.asarray(cell, dtype=np.float64).reshape(3, 3))))
    if vol <= 0 or nat <= 1:
        return 0.0
    rho = nat / vol
    return nat * rho * 4.0 / 3.0 * math.pi * cutoff ** 3


def predicted_pair_bytes(nat: int, cell, cutoff: float, bytes_per_pair: int = BYTES_PER_PAIR) -> float:
    return predicted_pairs(nat, cell, cutoff) * bytes_per_pair


def partition(costs: Sequence[float], nparts: int) -> List[List[int]]:
    """Greedy longest-processing-time partition of item indices into nparts
    lists with balanced total cost.  Deterministic (ties by index)."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    order = sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k))
    heap = [(0.0, p) for p in range(nparts)]
    heapq.heapify(heap)
    parts: List[List[int]] = [[] for _ in range(nparts)]
    for k in order:
        load, p = heapq.heappop(heap)
        parts[p].append(k)
        heapq.heappush(heap, (load + float(costs[k]), p))
    return [sorted(p) for p in parts]


def rank_systems(costs: Sequence[float], rank: int, world: int) -> List[int]:
    """The systems this rank owns."""
    return partition(costs, world)[rank]


def max_over_ranks(value: float) -> float:
    """Max of a scalar over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
