"""Sharding of independent units across ranks (one process per GPU).

The single-state circuits do not shard (one state vector; QuEST's pairwise
chunk exchange, QuEST_cpu_distributed.c:498-560, is out of scope), so they
run as replicas.  Independent units -- the swap tests of a QKMeans distance
batch, Trotter instances -- are dealt to ranks with no device collective:
each rank runs its share on its own GPU, and only host scalars (the
per-unit results, the step time) cross ranks, over torch.distributed (gloo
on the host).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np


def shard_units(costs: Sequence[float], world: int, rank: int) -> np.ndarray:
    """Indices of the units rank `rank` of `world` takes: units sorted by cost
    (largest first) and dealt greedily to the least-loaded rank, so the
    per-rank totals differ by at most the largest unit.  Deterministic: every
    rank computes the same assignment without communicating."""
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return np.nonzero(owner == rank)[0]


def swap_test_cost(dim_log2: np.ndarray) -> np.ndarray:
    """Relative cost of a swap test on vectors of length 2^d: the explicit
    state has 2^(2d+1) amplitudes."""
    return np.ldexp(1.0, 2 * np.asarray(dim_log2, dtype=np.int64) + 1)


def trotter_instance_cost(steps: Sequence[int], order: Sequence[int]) -> np.ndarray:
    """Relative cost of a Trotter instance (same register size): its fused
    passes grow with the Pauli exponentials applied, steps x the exponentials
    per step.  Per step, order 1 applies every term once and order 2 twice
    (the symmetrised product); order 2k applies five order-(2k-2) products
    (QuEST_common.c:800-820), so 2 x 5^(k-1) times."""
    steps = np.asarray(steps, dtype=np.float64)
    order = np.asarray(order, dtype=np.int64)
    return steps * np.where(order == 1, 1.0, 2.0 * np.power(5.0, np.maximum(order // 2 - 1, 0)))


def gather_to_rank0(indices: np.ndarray, values: np.ndarray, total: int, world: int):
    """Assemble the per-unit results of all ranks into one array on rank 0
    (None on the others).  world == 1 needs no process group."""
    if world == 1:
        out = np.full(total, np.nan)
        out[indices] = values
        return out
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(indices), np.asarray(values)))
    if dist.get_rank() != 0:
        return None
    out = np.full(total, np.nan)
    for idx, val in parts:
        out[idx] = val
    return out


def max_over_ranks(value: float, world: int) -> float:
    """The largest of the ranks' values (the step time of a sharded job)."""
    if world == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
