"""Partition of k-point work over ranks, and the gather of the results (one process per GPU).

k-points are independent, so a multi-GPU band structure is a partition of the k list, a local solve
per rank and a gather to the owner. The reference does this for its dielectric function with MPI
(apps/epsilon.cpp:250-259: contiguous blocks, the first nk % P ranks one k-point more;
epsilon.cpp:298-320: MPI_Gather of the sizes, MPI_Gatherv of the payloads to rank 0). Here the same
partition is kept and the gather runs over torch.distributed (NCCL between GPUs, gloo on CPU), with
the variable sizes handled by padding to the largest block. For uneven work (several materials,
cutoffs and SOC settings in one job) `cost_bins` balances groups by their estimated cost instead of
their k-point counts.

There is no collective in the solve itself: each rank's kernels only touch its own block.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def block_counts(nk: int, world: int) -> np.ndarray:
    """k-points per rank: nk // world each, one more for the first nk % world ranks."""
    if world <= 0:
        raise ValueError("world size must be positive")
    if nk < 0:
        raise ValueError("negative number of k-points")
    base, rem = divmod(nk, world)
    return np.array([base + (1 if p < rem else 0) for p in range(world)], dtype=np.int64)


def block_offsets(counts: Sequence[int]) -> np.ndarray:
    """Start index of each rank's block (exclusive prefix sum of the counts)."""
    c = np.asarray(counts, dtype=np.int64)
    return np.concatenate([[0], np.cumsum(c)[:-1]]).astype(np.int64)


def shard_range(nk: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's block of a list of nk k-points."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    c = block_counts(nk, world)
    o = block_offsets(c)
    return int(o[rank]), int(o[rank] + c[rank])


def solve_cost(n: int, nk: int, nb: int = 16) -> float:
    """Relative cost of solving nk matrices of order n for nb bands: the O(n^3) reduction plus the
    O(n^2 nb) vector work, per k-point."""
    return float(nk) * (n ** 3 + 4.0 * n * n * nb)


def cost_bins(costs: Sequence[float], world: int) -> list[list[int]]:
    """Assigns work items (e.g. one (material, cutoff, SOC) group each) to ranks, largest first onto
    the least-loaded rank (longest-processing-time rule: the makespan is within 4/3 of optimal).
    Returns the item indices of each rank, each list in increasing order."""
    if world <= 0:
        raise ValueError("world size must be positive")
    load = np.zeros(world)
    bins: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda q: (-float(costs[q]), q)):
        r = int(np.argmin(load))
        bins[r].append(i)
        load[r] += float(costs[i])
    return [sorted(b) for b in bins]


def gather_blocks(local: np.ndarray, counts: Sequence[int], dst: int = 0, group=None, device=None):
    """Gathers each rank's block of rows (local.shape[0] == counts[rank]) into the full array on
    rank dst, in rank order; returns None on the other ranks. Every rank passes the same counts and
    the same trailing shape and dtype."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    counts = [int(c) for c in counts]
    if len(counts) != world:
        raise ValueError(f"{len(counts)} block counts for a world of {world}")
    if local.shape[0] != counts[rank]:
        raise ValueError(f"rank {rank} holds {local.shape[0]} rows, its block has {counts[rank]}")
    mx = max(counts) if counts else 0
    tail = tuple(local.shape[1:])
    pad = np.zeros((mx,) + tail, dtype=local.dtype)
    pad[: local.shape[0]] = local
    t = torch.from_numpy(pad)
    if device is not None:
        t = t.to(device)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    if rank != dst:
        return None
    return np.concatenate([p.cpu().numpy()[:c] for p, c in zip(parts, counts)], axis=0)


def distributed_solve(solve: Callable[[np.ndarray], np.ndarray], k: np.ndarray, dst: int = 0, group=None,
                      device=None):
    """Runs solve on this rank's block of the k list and gathers the rows on rank dst (None elsewhere).
    solve maps a (count, 3) array of k-points to a (count, ...) result array."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    counts = block_counts(len(k), world)
    a, b = shard_range(len(k), rank, world)
    local = np.ascontiguousarray(solve(np.ascontiguousarray(k[a:b])))
    return gather_blocks(local, counts, dst=dst, group=group, device=device)
