"""Sharding products across GPUs: one process per GPU, no data-path collective.

Every product is independent, so a batch partitions across ranks with no
exchange: each rank computes its share on its own GPU with its own tables,
and only the results travel, to the host of the rank that asked for them.
The reference runs on one GPU and has no multi-GPU path; this follows the
batch split of its batched plugin (native-batched/solve.cu:200-244) one level
up, over GPUs instead of slots.

  plan(costs, world)            -> list of product indices per rank
  cost(N, W)                    -> relative work of one product
  run_sharded(items, fn, group) -> results of every item, on every rank (or on dst)
"""
from __future__ import annotations

import heapq
from typing import Callable, Sequence


def cost(N: int, W: int) -> float:
    """Relative work of one product: N coefficients times P primes, P ~ (2W + log2 N) / 31."""
    return float(N) * (2 * W + N.bit_length() + 2)


def plan(costs: Sequence[float], world: int) -> list[list[int]]:
    """Assigns every product to exactly one rank, balancing summed cost.

    Longest-processing-time first (a 4/3-approximation of the best split),
    deterministic: ties go to the lower rank, and each rank's indices come
    back in ascending order.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    shares: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def run_sharded(items: Sequence, fn: Callable, costs: Sequence[float] | None = None, group=None,
                dst: int | None = None) -> list | None:
    """Runs fn(item) for this rank's share of `items` and gathers the results.

    With torch.distributed initialised, rank r computes plan(costs, world)[r];
    the results (host objects, e.g. numpy arrays) are gathered in item order
    on every rank (dst None) or on rank dst only (other ranks get None).
    Without torch.distributed, runs everything locally.
    """
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [fn(x) for x in items]
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    shares = plan(costs if costs is not None else [1.0] * len(items), world)
    mine = {i: fn(items[i]) for i in shares[rank]}
    if dst is None:
        gathered = [None] * world
        dist.all_gather_object(gathered, mine, group=group)
    else:
        gathered = [None] * world if rank == dst else None
        dist.gather_object(mine, gathered, dst=dst, group=group)
        if rank != dst:
            return None
    out = [None] * len(items)
    for part in gathered:
        for i, v in part.items():
            out[i] = v
    return out
