"""Autotuner for the launch parameters of the hafnian DP kernel.

Each DP warp keeps its items' DP-state (F) ring in a per-warp scratch slice
sized for the largest program of its launch (the class-pair values come
straight from the site's Sigma).  The
items are split into two launches by table size (programs with at most
`small_entries` table entries run with small slices), and the number of
resident warps is capped by a scratch budget.  The best split point,
residency and budget depend on the workload (d, chi, photon numbers); the
tuner times the DP kernel class with the library's CUDA-event profiler over
full builds and keeps the fastest setting on the handle.

    from bosonsupremacy_gb300 import autotune
    best, table = autotune.tune_dp(sq_cov, d, chi)   # sets the knobs
    best, table = autotune.tune_batch(sq_covs, ds, chis)   # many instances per call
"""
from __future__ import annotations

import ctypes as C
import itertools
from typing import Dict, Iterable, Tuple

import torch

from . import _lib
from .pipeline import build_mps, build_mps_batch

KNOBS = {
    "blocks_per_sm": _lib.TUNE_DP_BLOCKS_PER_SM,
    "l1_carveout": _lib.TUNE_DP_L1_CARVEOUT,
    "small_entries": _lib.TUNE_DP_SMALL_ENTRIES,
    "small_blocks": _lib.TUNE_DP_SMALL_BLOCKS,
    "scratch_mib": _lib.TUNE_DP_SCRATCH_MIB,
    "fp64_blocks": _lib.TUNE_DP_FP64_BLOCKS,
    "factor_threads": _lib.TUNE_FACTOR_THREADS,
    "gemm_kernel": _lib.TUNE_GEMM_KERNEL,
    "dp_quantum": _lib.TUNE_DP_QUANTUM,
    "dp_hold": _lib.TUNE_DP_HOLD,
    "right_pct": _lib.TUNE_RIGHT_PCT,
    "left_pct": _lib.TUNE_LEFT_PCT,
    "factor_dual": _lib.TUNE_FACTOR_DUAL,
    "dp_order": _lib.TUNE_DP_ORDER,
}


def get_knobs(device: int = 0) -> Dict[str, int]:
    lib = _lib.load()
    h = _lib.Handle.get(device)
    out = {}
    for name, key in KNOBS.items():
        v = C.c_int()
        _lib.check(lib.bsg_tune_get(h.h, key, C.byref(v)), "bsg_tune_get")
        out[name] = v.value
    return out


def set_knobs(device: int = 0, **values: int) -> None:
    lib = _lib.load()
    h = _lib.Handle.get(device)
    for name, v in values.items():
        _lib.check(lib.bsg_tune_set(h.h, KNOBS[name], int(v)), "bsg_tune_set")


def dp_time_ms(sq_cov, d: int, chi: int, precision: str = "split", device: int = 0, reps: int = 1,
               out=None) -> float:
    """Mean DP-kernel time (ms) of `reps` full builds."""
    lib = _lib.load()
    h = _lib.Handle.get(device)
    lib.bsg_profile_reset(h.h)
    lib.bsg_profile_enable(h.h, 1)
    try:
        for _ in range(reps):
            build_mps(sq_cov, d, chi, precision=precision, device=device, out=out)
        torch.cuda.synchronize()
        ms, n, w = C.c_double(), C.c_int64(), C.c_double()
        _lib.check(lib.bsg_profile_read(h.h, _lib.K_DP, C.byref(ms), C.byref(n), C.byref(w)), "bsg_profile_read")
    finally:
        lib.bsg_profile_enable(h.h, 0)
    return ms.value / max(1, reps)


def tune_dp(sq_cov, d: int, chi: int, precision: str = "split", device: int = 0,
            grid: Dict[str, Iterable[int]] | None = None, reps: int = 1
            ) -> Tuple[Dict[str, int], Dict[Tuple[int, ...], float]]:
    """Times every point of `grid` (knob name -> values; knobs left out keep
    their current value) after a warm-up build, leaves the fastest on the
    handle and returns (best knobs, {values tuple: ms})."""
    if grid is None:
        grid = {"blocks_per_sm": (4, 8), "small_entries": (0, 64, 256), "scratch_mib": (2048, 8192)}
    M = len(sq_cov) // 2
    dtype = torch.complex64
    out = [torch.empty(chi, chi, d, dtype=dtype, device=torch.device("cuda", device)) for _ in range(M)]
    build_mps(sq_cov, d, chi, precision=precision, device=device, out=out)  # programs, workspaces
    names = list(grid)
    table = {}
    for values in itertools.product(*(tuple(grid[n]) for n in names)):
        set_knobs(device, **dict(zip(names, values)))
        table[values] = dp_time_ms(sq_cov, d, chi, precision, device, reps=reps, out=out)
    best = min(table, key=table.get)
    set_knobs(device, **dict(zip(names, best)))
    return dict(zip(names, best)), table


def tune_batch(sq_covs, ds, chis, precision: str = "split", device: int = 0,
               grid: Dict[str, Iterable[int]] | None = None, reps: int = 2
               ) -> Tuple[Dict[str, int], Dict[Tuple[int, ...], float]]:
    """The same search for the batched build of many independent instances
    (bsg_build_mps_batch), timed as whole batched builds with CUDA events:
    the table-size split of the DP's two launches (`small_entries`: which
    partition programs run with small per-warp tables), the work quantum of
    its yielding launches (`dp_quantum`: how many program transitions a warp
    runs before its block gives the SM back) and the resident blocks.  Leaves
    the fastest setting on the handle and returns (best knobs, {values: ms})."""
    if grid is None:
        grid = {"small_entries": (0, 64, 256), "dp_quantum": (1, 2, 8), "blocks_per_sm": (4, 8)}
    dev = torch.device("cuda", device)
    Ms = [len(q) // 2 for q in sq_covs]
    outs = [[torch.empty(c, c, d, dtype=torch.complex64, device=dev) for _ in range(M)]
            for M, d, c in zip(Ms, ds, chis)]
    sqs = [torch.as_tensor(q).to(dev) for q in sq_covs]
    build_mps_batch(sqs, ds, chis, precision=precision, device=device, outs=outs)  # programs, workspaces
    stream = torch.cuda.current_stream(dev)
    names = list(grid)
    table = {}
    for values in itertools.product(*(tuple(grid[n]) for n in names)):
        set_knobs(device, **dict(zip(names, values)))
        build_mps_batch(sqs, ds, chis, precision=precision, device=device, outs=outs)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            build_mps_batch(sqs, ds, chis, precision=precision, device=device, outs=outs)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        table[values] = e0.elapsed_time(e1) / reps
    best = min(table, key=table.get)
    set_knobs(device, **dict(zip(names, best)))
    return dict(zip(names, best)), table
