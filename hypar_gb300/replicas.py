"""Runs over several GPUs of one node: one process per GPU, no data exchanged.

HyPar splits one grid over MPI ranks with a three-cell halo exchange per
right-hand side (src/MPIFunctions/MPIExchangeBoundariesnD.c:42-173); this
package computes a grid on one GPU and has no halo exchange.  Over N GPUs it
therefore runs either N independent replicas of a problem or, for an ensemble,
disjoint subsets of the members: HyPar's ensemble members are independent
simulations that share only dt and solver.inp (src/Simulation/ReadInputs.c:189-206),
so a member never needs data from another GPU.  The one collective is the
maximum over ranks of a timed interval (and a barrier around it).
"""

from __future__ import annotations

from typing import List, Sequence


def shard_members(cells: Sequence[int], world_size: int) -> List[List[int]]:
    """Partition ensemble members over `world_size` ranks by their cell counts.

    Longest-processing-time greedy: members in decreasing size (ties by index)
    each go to the rank with the smallest load so far (ties to the lower rank).
    Deterministic, so every rank computes the same partition without
    communication.  Returns, per rank, its member indices in increasing order;
    a rank may receive none when there are fewer members than ranks.
    """
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    if any(int(c) < 0 for c in cells):
        raise ValueError("cell counts must be non-negative")
    order = sorted(range(len(cells)), key=lambda k: (-int(cells[k]), k))
    load = [0] * world_size
    parts: List[List[int]] = [[] for _ in range(world_size)]
    for k in order:
        r = min(range(world_size), key=lambda j: (load[j], j))
        parts[r].append(k)
        load[r] += int(cells[k])
    return [sorted(p) for p in parts]


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The maximum of `x` over the ranks of the default process group (`x` itself
    when `dist` is None).  `device` is where the reduction tensor lives: a CUDA
    device for NCCL, None (CPU) for gloo."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world_size: int, seconds: float) -> float:
    """Whole-job throughput of replicas: every rank processed `units_per_rank`
    units and the job took the slowest rank's `seconds`."""
    if seconds <= 0.0:
        raise ValueError("seconds must be positive")
    return world_size * float(units_per_rank) / seconds
