"""Sharding of an ECP job over ranks (one process per GPU).

Every (shell pair, ECP centre) unit is independent, so ranks split the ECP
centres round-robin and need no communication while computing; the one
exchange is the final sum of the partial AO matrices (each rank holds the
contribution of its centres), done with torch.distributed.all_reduce.
"""
from __future__ import annotations

import numpy as np

from .workloads import EcpSystem


def centres_of_rank(s: EcpSystem, rank: int, world: int) -> list[int]:
    """ECP atoms of this rank: the rank-th, (rank+world)-th, ... ECP atom."""
    centres = [a for a in range(s.n_atoms) if s.shellsECP[a] > 0]
    return centres[rank::world]


def shard(s: EcpSystem, rank: int, world: int) -> EcpSystem:
    """The rank's part of the job: same geometry and basis, its ECP centres only."""
    return s.subset(centres=centres_of_rank(s, rank, world))


def all_reduce_matrix(I: np.ndarray) -> np.ndarray:
    """Sums the partial matrices of all ranks (in place, returns I)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(I)
    if dist.get_backend() == "nccl":
        g = t.cuda()
        dist.all_reduce(g)
        t.copy_(g.cpu())
    else:
        dist.all_reduce(t)
    return I


def distributed_get_integrals(s: EcpSystem, compute, rank: int, world: int) -> np.ndarray:
    """Full ECP matrix on every rank: compute(shard) then one all-reduce.
    `compute(system) -> matrix` is the per-rank engine call."""
    I = compute(shard(s, rank, world))
    return all_reduce_matrix(np.ascontiguousarray(I))
