"""Multi-rank host logic.

The MPS build partitions naturally: cut c depends only on the covariance,
site i only on cuts i-1 and i (MPS_cpu.py:463-472).  Ranks therefore need no
collective on the data path.  The reference spreads the same work one rank
per mode with MPI work stealing (distributed_MPS.py:57-311); here a rank owns
a contiguous site range balanced by estimated work, builds the cuts its
sites read, and only the timing is reduced.  bench.py runs independent
instances per rank (weak scaling).
"""
from __future__ import annotations

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
