"""Multi-GPU execution of independent units (sectors, disorder realisations, SIAM instances).

The reference runs everything in one process (cmpy/exactdiag.py:24-43 loops over sectors).
Its units are independent, so on several GPUs each rank solves a shard of the units and the
only cross-rank step is a host-side reduction of the results — no collective touches the
data path. One process per GPU; ranks come from torch.distributed (NCCL on GPUs, gloo on
CPU for tests).
"""

from __future__ import annotations

import heapq
from typing import Any, Callable, Iterable, Sequence

__all__ = ["shard_units", "compute_groundstate_distributed", "gather_results"]


def shard_units(costs: Sequence[float], world: int) -> list[list[int]]:
    """Longest-processing-time assignment of units (by cost, e.g. sector dimension) to ranks.
    Deterministic: ties broken by unit index, then rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    for r in range(world):
        out[r].sort()
    return out


def _dist():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        return dist
    return None


def gather_results(local: dict, dist=None) -> dict:
    """Union of per-rank {unit_index: result} dicts on every rank (all_gather_object)."""
    dist = dist or _dist()
    if dist is None:
        return dict(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, local)
    merged: dict = {}
    for p in parts:
        merged.update(p)
    return merged


def compute_groundstate_distributed(model, solve: Callable[[Any, int, int], tuple[float, Any]] | None = None,
                                    fillings: Iterable[tuple[int, int]] | None = None, dist=None):
    """Ground state over all (n_up, n_dn) sectors, sharded over the ranks of the current
    process group. `solve(model, n_up, n_dn) -> (energy, state)` defaults to the device
    solver. Returns (energy, n_up, n_dn, state-or-None on non-owning ranks)."""
    from math import comb

    dist = dist or _dist()
    rank = dist.get_rank() if dist else 0
    world = dist.get_world_size() if dist else 1
    if fillings is None:
        fillings = list(model.basis.iter_fillings())
    fillings = list(fillings)
    if solve is None:
        from .exactdiag import groundstate_sector

        solve = groundstate_sector
    n = model.num_sites
    costs = [comb(n, a) * comb(n, b) for a, b in fillings]
    mine = shard_units(costs, world)[rank]
    local = {}
    states = {}
    for i in mine:
        e, st = solve(model, *fillings[i])
        local[i] = float(e)
        states[i] = st
    energies = gather_results(local, dist)
    best = min(energies, key=lambda i: (energies[i], i))
    nu, nd = fillings[best]
    return energies[best], nu, nd, states.get(best)
