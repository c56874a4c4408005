"""Drop-in for kron_cpu.py: per-cut Schmidt spectra on the GPU.

    python -m bosonsupremacy_gb300.kron --d D --chi CHI --dir ROOT/

Same flags (kron_cpu.py:11-19), same inputs (ROOT/sq_cov.npy, ROOT/cov.npy)
and the same outputs in ROOT/d_{D}_chi_{CHI}/ (kron_cpu.py:134-153):
``active_kron_sites.npy`` and, for every cut i = 0..M-2 (between modes i and
i+1), ``res_i.npy`` (Schmidt weights, descending), ``num_i.npy`` (int8 Fock
labels [kept, M-1-i]) and ``S_i.npy`` (Williamson symplectic of modes
i+1..M-1, xxpp).  ``res_i`` is saved as float64 (the FP64-promoted form);
``--ref-dtypes`` saves it as float16 like kron_cpu.py:127.

The Williamson basis (and so ``S_i`` and the column order of ``num_i``)
differs from scipy's by a symplectic-orthogonal gauge per mode and orders
modes by symplectic eigenvalue; MPS_cpu.py and bosonsupremacy_gb300.mps both
consume these files unchanged, and every physical output is gauge invariant.
"""
from __future__ import annotations

import argparse
import os
import time
from typing import List, Tuple

import numpy as np
import torch

from . import dist, ops

CUT_TOL = 1e-12  # kron_cpu.py:95 err_tol


def thermal_photons(nth, cutoff=20):
    """Geometric photon-number distribution of a thermal mode (kron_cpu.py:92-93)."""
    return 1 / (nth + 1) * (nth / (nth + 1)) ** np.arange(cutoff)


def get_cumsum_kron_range(sq_cov: np.ndarray, d: int, chi: int, c0: int, c1: int,
                          device: int = 0) -> List[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """(res, num, S) of cuts c0 .. c1-1, as kron_cpu.py's main loop produces them."""
    M = sq_cov.shape[0] // 2
    if c1 <= c0:
        return []
    res, num, S, kept = ops.cut_spectra(sq_cov, d, chi, L0=c0 + 1, n_cuts=c1 - c0, err_tol=CUT_TOL, device=device)
    res, num, S, kept = res.cpu().numpy(), num.cpu().numpy(), S.cpu().numpy(), kept.cpu().numpy()
    out = []
    for j, c in enumerate(range(c0, c1)):
        k = M - 1 - c
        out.append((res[j, : kept[j]].copy(), num[j, : kept[j], :k].copy(), S[j, : 2 * k, : 2 * k].copy()))
    return out


def get_cumsum_kron_all(sq_cov: np.ndarray, d: int, chi: int, device: int = 0) -> List[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """(res, num, S) of every cut, as kron_cpu.py's main loop produces them."""
    return get_cumsum_kron_range(sq_cov, d, chi, 0, sq_cov.shape[0] // 2 - 1, device=device)


def get_cumsum_kron(sq_cov: np.ndarray, L: int, chi: int = 100, max_dim: int = 10 ** 5, cutoff: int = 6,
                    err_tol: float = 1e-12, device: int = 0):
    """Single-cut form of kron_cpu.py:95 (returns res, num, S for the cut
    before mode L).  ``max_dim`` is accepted for signature compatibility:
    keeping the top chi per step selects the same set (see bsg_cuts.cu)."""
    M = sq_cov.shape[0] // 2
    res, num, S, kept = ops.cut_spectra(sq_cov, cutoff, chi, L0=L, n_cuts=1, err_tol=err_tol, device=device)
    k = M - L
    kk = int(kept[0].item())
    return res[0, :kk].cpu().numpy(), num[0, :kk, :k].cpu().numpy(), S[0, : 2 * k, : 2 * k].cpu().numpy()


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--d", type=int, help="Maximum number of photons per mode before displacement - 1.")
    p.add_argument("--chi", type=int, help="Bond dimension.")
    p.add_argument("--dir", type=str, help="Root directory.", default=0)
    p.add_argument("--ref-dtypes", action="store_true", help="save res as float16 like kron_cpu.py")
    p.add_argument("--device", type=int, default=None, help="GPU (default: torchrun's LOCAL_RANK, else 0)")
    args = p.parse_args(argv)
    d, chi, rootdir = args.d, args.chi, args.dir
    path = rootdir + f"d_{d}_chi_{chi}/"
    sq_cov = np.load(rootdir + "sq_cov.npy")
    cov = np.load(rootdir + "cov.npy")
    M = len(cov) // 2
    # under torchrun each rank writes the files of its own contiguous cut range
    rank, world, local = dist.rank_world()
    device = args.device if args.device is not None else local % max(1, torch.cuda.device_count())
    c0, c1 = dist.shard_cuts(M, world)[rank] if world > 1 else (0, M - 1)
    os.makedirs(path, exist_ok=True)
    if rank == 0:
        np.save(path + "active_kron_sites.npy", np.zeros(M - 1, dtype="int32"))
    t0 = time.time()
    cuts = get_cumsum_kron_range(sq_cov, d, chi, c0, c1, device=device)
    for c, (res, num, S) in zip(range(c0, c1), cuts):
        print(c, np.sum(res))
        np.save(path + f"res_{c}.npy", res.astype("float16") if args.ref_dtypes else res)
        np.save(path + f"num_{c}.npy", num.astype("int8"))
        np.save(path + f"S_{c}.npy", S)
    print(f"cuts: {c1 - c0} in {time.time() - t0:.3f} s")


if __name__ == "__main__":
    main()
