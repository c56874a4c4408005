"""Multi-rank host logic.

The MPS build partitions naturally: cut c depends only on the covariance,
site i only on cuts i-1 and i (MPS_cpu.py:463-472).  Ranks therefore need no
collective on the data path.  The reference spreads the same work one rank
per mode with MPI work stealing (distributed_MPS.py:57-311); here a rank owns
a contiguous range: the ``kron`` and ``mps`` command-line steps, launched
with torchrun, each write their own ranks' cut and site files (the
reference's file contract), and bench.py runs independent instances per rank
(weak scaling), reducing only the timing.
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple


def site_cost(M: int, i: int) -> float:
    """Relative cost of site i: items ~ chi^2 d everywhere except the two ends,
    Sigma ~ (M - i)^3."""
    if i == 0 or i == M - 1:
        return 0.05
    return 1.0 + 0.2 * ((M - i) / M) ** 3


def shard_sites(M: int, world: int, costs: Sequence[float] = None) -> List[Tuple[int, int]]:
    """Contiguous [start, stop) site ranges, one per rank, with near-equal cost."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    costs = list(costs) if costs is not None else [site_cost(M, i) for i in range(M)]
    total = sum(costs)
    out, start, acc = [], 0, 0.0
    for r in range(world):
        target = total * (r + 1) / world
        stop = start
        while stop < M and (acc + costs[stop] <= target or stop == start) and M - stop > world - r - 1:
            acc += costs[stop]
            stop += 1
        if r == world - 1:
            while stop < M:
                acc += costs[stop]
                stop += 1
        out.append((start, stop))
        start = stop
    return out


def rank_world() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from torchrun's environment; (0, 1, 0) without it."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def cut_cost(M: int, c: int) -> float:
    """Relative cost of cut c (L = c + 1 left modes, k = M - 1 - c right
    modes): the eigen-solve of the 2 min(L, k) core plus the pivoted pairing
    of the 2 (k - L) vacuum modes among 2k-vectors, weighted as measured on
    the M=144 build (cut 0 and cut 72 both take ~30 ms)."""
    L, k = c + 1, M - 1 - c
    return 8.7 * float(2 * min(L, k)) ** 3 + 0.96 * 8.0 * float(max(0, k - L)) ** 2 * k


def shard_cuts(M: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous [start, stop) cut ranges, one per rank, with near-equal cost."""
    return shard_sites(M - 1, world, [cut_cost(M, c) for c in range(M - 1)])


def cuts_needed(site_range: Tuple[int, int], M: int) -> Tuple[int, int]:
    """[first, stop) cut indices the sites of a range read (cut c lies between modes c and c+1)."""
    a, b = site_range
    return max(0, a - 1), min(M - 1, b)


def reduce_max(value: float) -> float:
    """Max over ranks (the bench's timing rule); identity without a process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return value
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
