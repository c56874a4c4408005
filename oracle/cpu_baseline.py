"""ORACLE -- test/benchmark infrastructure only, never the product.

CPU baseline of the reference's MPS construction (kron_cpu.py + MPS_cpu.py,
FP64-promoted restatement in ``oracle.reference_mps``) timed on a BOUNDED
sample of a workload and extrapolated to the full build.  Used only by
bench.py's cpu_baseline leg and its ``--impl reference`` arm.

Model of the reference's own loop structure (MPS_cpu.py:384-525):
  * every site runs ``williamson(sq_cov)`` (MPS_cpu.py:395) and one
    ``get_U2_sq_U1`` (Bloch-Messiah, :481);
  * every (j, photon sector `size`) group of a site is one A_elem call on a
    batch of B items of order n = j + size (:486-519); A_elem gathers
    (Sigma_select, cost ~ B n^2) and runs the batched recursion, whose Python
    statement count is the recursion's complex-MAC count C(n) (each statement
    a numpy op over the batch), so a group costs a*C(n) + b*C(n)*B + g*B*n^2 + o;
  * kron: every cut runs (k-1) product/argsort steps at max_dim = 1e5
    (kron_cpu.py:109-119), roughly constant per step once saturated.
The coefficients are fitted from timed samples of this machine; the group
sizes are the workload's exact ones (from its cut data).
"""
from __future__ import annotations

import functools
import time
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import reference_mps as R


@functools.lru_cache(maxsize=None)
def recursion_macs(n: int) -> int:
    """Complex multiply-adds of hafnian() at order n (MPS_cpu.py:117-187)."""
    if n % 2 or n < 4:
        return 0
    if n == 4:
        return 3
    h = n // 2

    @functools.lru_cache(maxsize=None)
    def C(s):
        if s == 0:
            return 0
        return 2 * C(s - 2) + ((s - 2) * (s - 3) // 2) * h * (h + 1) + h * (h + 1) // 2

    return C(n)


def group_sizes(cuts: Sequence[tuple], M: int, d: int, err_tol: float = 1e-10) -> List[Tuple[int, int]]:
    """(n, B) of every A_elem call the reference's site loop makes."""
    return [g for site in site_group_sizes(cuts, M, d, err_tol) for g in site]


def site_group_sizes(cuts: Sequence[tuple], M: int, d: int, err_tol: float = 1e-10) -> List[List[Tuple[int, int]]]:
    """Per site, (n, B) of every A_elem call of that site (MPS_cpu.py:486-519)."""
    per_site = []
    for site in range(M):
        out: List[Tuple[int, int]] = []
        if site == 0:
            res, num, _ = cuts[0]
            keep = res > err_tol
            sums = num[keep].reshape(int(keep.sum()), -1).sum(1)
            vals, cnts = np.unique(sums, return_counts=True)
            for j in range(d):
                out += [(j + int(v), int(c)) for v, c in zip(vals, cnts)]
        elif site == M - 1:
            num_pre = cuts[site - 1][1]
            sums = num_pre.reshape(num_pre.shape[0], -1).sum(1)
            vals, cnts = np.unique(sums, return_counts=True)
            for j in range(d):
                out += [(j + int(v), int(c)) for v, c in zip(vals, cnts) if not (j == 0 and v == 0)]
        else:
            res, num, _ = cuts[site]
            keep = res > err_tol
            ls = num[keep].reshape(int(keep.sum()), -1).sum(1)
            rs = cuts[site - 1][1].reshape(cuts[site - 1][1].shape[0], -1).sum(1)
            lv, lc = np.unique(ls, return_counts=True)
            rv, rc = np.unique(rs, return_counts=True)
            tot: Dict[int, int] = {}
            for a, ca in zip(lv, lc):
                for b, cb in zip(rv, rc):
                    tot[int(a + b)] = tot.get(int(a + b), 0) + int(ca * cb)
            for j in range(d):
                out += [(j + s, c) for s, c in tot.items() if not (j == 0 and s == 0)]
        per_site.append(out)
    return per_site


def _time_group(Sigma, n: int, B: int, rng) -> float:
    idx = rng.integers(0, Sigma.shape[0], size=(B, n)).astype(np.int32)
    den = np.ones(B)
    t0 = time.perf_counter()
    R.A_elem(Sigma, idx, den)
    return time.perf_counter() - t0


def fit_site_model(Sigma: np.ndarray, rng, budget_s: float = 8.0) -> Dict[str, float]:
    """Fit a, b (per recursion statement, per statement-item), g (gather per
    item*n^2) and o (per call) from timed A_elem calls."""
    rows, ts = [], []
    t_start = time.perf_counter()
    for n in (6, 8, 10, 12):
        for B in (8, 512):
            if time.perf_counter() - t_start > budget_s:
                break
            t = min(_time_group(Sigma, n, B, rng) for _ in range(2))
            rows.append([recursion_macs(n), recursion_macs(n) * B, B * n * n, 1.0])
            ts.append(t)
    for n, B in ((1, 20000), (3, 20000), (2, 64)):  # gather-only and overhead points
        t = min(_time_group(Sigma, n, B, rng) for _ in range(2))
        rows.append([recursion_macs(n), recursion_macs(n) * B, B * n * n, 1.0])
        ts.append(t)
    A = np.array(rows, dtype=float)
    coef, *_ = np.linalg.lstsq(A, np.array(ts), rcond=None)
    coef = np.maximum(coef, 0.0)
    return {"a": coef[0], "b": coef[1], "g": coef[2], "o": coef[3]}


def estimate_full_build(sq_cov: np.ndarray, d: int, chi: int, cuts: Sequence[tuple], budget_s: float = 20.0,
                        seed: int = 0) -> Dict[str, float]:
    """Extrapolated wall time of kron_cpu.py + MPS_cpu.py on this host."""
    rng = np.random.default_rng(seed)
    M = sq_cov.shape[0] // 2
    t_sample0 = time.perf_counter()
    # kron: one middle cut at the reference's max_dim = 1e5
    Lm = max(1, M // 2)
    t0 = time.perf_counter()
    R.get_cumsum_kron(sq_cov, Lm, chi=chi, max_dim=10 ** 5, cutoff=d)
    t_cut = time.perf_counter() - t0
    steps_mid = max(1, M - Lm - 1)
    steps_all = sum(max(0, M - L - 1) for L in range(1, M))
    t_kron = t_cut / steps_mid * steps_all
    # per-site dense work: williamson of the full state and one Bloch-Messiah
    t0 = time.perf_counter()
    S_full = R.williamson(sq_cov)[1]
    t_will = time.perf_counter() - t0
    site = max(1, min(M - 2, M // 2))
    t0 = time.perf_counter()
    U2, sq, U1 = R.get_U2_sq_U1(cuts[site][2], cuts[site - 1][2])
    Sigma = R.get_Sigma(U2, sq, U1)
    t_bm = time.perf_counter() - t0
    # hafnian groups
    model = fit_site_model(Sigma, rng, budget_s=max(2.0, budget_s - (time.perf_counter() - t_sample0)))
    groups = group_sizes(cuts, M, d)
    t_haf = 0.0
    for n, B in groups:
        C = recursion_macs(n)
        t_haf += model["a"] * C + model["b"] * C * B + model["g"] * B * n * n + model["o"]
    total = t_kron + M * (t_will + t_bm) + t_haf
    return {
        "build_s": total,
        "kron_s": t_kron,
        "dense_s": M * (t_will + t_bm),
        "hafnian_s": t_haf,
        "groups": len(groups),
        "items": int(sum(B for _, B in groups)),
        "sample_s": time.perf_counter() - t_sample0,
        "sites_per_s": M / total,
    }


# ---- all host cores ----------------------------------------------------------
# The reference's multi-process form (distributed_kron.py / distributed_MPS.py)
# gives each rank whole cuts and whole sites.  Here every host core runs the
# same timed sample at once (so the per-core costs include the memory and
# clock contention of a fully loaded host), and the cuts, then the sites, are
# spread over the cores longest first; the build time is the sum of the two
# makespans.


def _sample_worker(args) -> Dict[str, float]:
    sq_cov, S_l, S_r, d, chi, budget_s, seed = args
    rng = np.random.default_rng(seed)
    M = sq_cov.shape[0] // 2
    Lm = max(1, M // 2)
    t0 = time.perf_counter()
    R.get_cumsum_kron(sq_cov, Lm, chi=chi, max_dim=10 ** 5, cutoff=d)
    t_cut = time.perf_counter() - t0
    t0 = time.perf_counter()
    R.williamson(sq_cov)
    t_will = time.perf_counter() - t0
    t0 = time.perf_counter()
    U2, sq, U1 = R.get_U2_sq_U1(S_l, S_r)
    Sigma = R.get_Sigma(U2, sq, U1)
    t_bm = time.perf_counter() - t0
    model = fit_site_model(Sigma, rng, budget_s=budget_s)
    return dict(model, t_cut_step=t_cut / max(1, M - Lm - 1), t_will=t_will, t_bm=t_bm)


def _makespan(costs: Sequence[float], procs: int) -> float:
    """Longest-processing-time-first assignment of independent tasks."""
    load = [0.0] * max(1, procs)
    for c in sorted(costs, reverse=True):
        i = min(range(len(load)), key=load.__getitem__)
        load[i] += c
    return max(load)


def estimate_full_build_parallel(sq_cov: np.ndarray, d: int, chi: int, cuts: Sequence[tuple], procs: int,
                                 budget_s: float = 20.0, seed: int = 0, timeout_s: float = 600.0) -> Dict[str, float]:
    """Extrapolated wall time of the reference's build on `procs` host cores
    (one process per core, one thread each).  Raises if a sample process
    fails or the samples exceed `timeout_s`."""
    import multiprocessing as mp
    import os
    from concurrent.futures import ProcessPoolExecutor

    M = sq_cov.shape[0] // 2
    site = max(1, min(M - 2, M // 2))
    jobs = [(sq_cov, cuts[site][2], cuts[site - 1][2], d, chi, budget_s, seed + 1000 * w) for w in range(procs)]
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"  # one thread per sample process (inherited at spawn)
    ex = ProcessPoolExecutor(max_workers=procs, mp_context=mp.get_context("spawn"))
    try:
        futs = [ex.submit(_sample_worker, j) for j in jobs]
        res = [f.result(timeout=timeout_s) for f in futs]
        ex.shutdown(wait=True)
    except BaseException:
        # do not wait for a stuck sample process: stop this pool's own workers
        procs_left = list(getattr(ex, "_processes", {}).values())
        ex.shutdown(wait=False, cancel_futures=True)
        for p in procs_left:
            if p.is_alive():
                p.kill()
        raise
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    med = {k: float(np.median([r[k] for r in res])) for k in res[0]}
    cut_costs = [med["t_cut_step"] * max(0, M - L - 1) for L in range(1, M)]
    site_costs = []
    for groups in site_group_sizes(cuts, M, d):
        t = med["t_will"] + med["t_bm"]
        for n, B in groups:
            C = recursion_macs(n)
            t += med["a"] * C + med["b"] * C * B + med["g"] * B * n * n + med["o"]
        site_costs.append(t)
    kron_s, mps_s = _makespan(cut_costs, procs), _makespan(site_costs, procs)
    total = kron_s + mps_s
    return {
        "build_s": total,
        "kron_s": kron_s,
        "mps_s": mps_s,
        "serial_s": float(sum(cut_costs) + sum(site_costs)),
        "largest_site_s": float(max(site_costs)),
        "procs": procs,
        "sites_per_s": M / total,
    }
