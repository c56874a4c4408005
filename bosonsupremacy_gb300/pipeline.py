"""Full MPS construction on one GPU: cut spectra -> Sigma per site -> Gamma
per site, with every tensor resident in HBM.

Mirrors the two reference steps kron_cpu.py (all cuts) and MPS_cpu.py (all
sites) with the same outputs: Gamma_i [chi, chi, d] (complex64 by default,
as MPS_cpu.py:397) and Lambda_i [chi] = sqrt(res_i) of the rows with
res_i > err_tol, zero padded (MPS_cpu.py:398, 415, 484).
"""
from __future__ import annotations

import dataclasses
import time
from typing import List, Optional

import numpy as np
import torch

from . import _lib, ops


@dataclasses.dataclass
class MPS:
    Gammas: List[torch.Tensor]      # M tensors [chi, chi, d]
    Lambdas: torch.Tensor           # [M-1, chi] float64
    res: torch.Tensor               # [M-1, chi] cut weights
    num: torch.Tensor               # [M-1, chi, M-1] labels
    S: torch.Tensor                 # [M-1, 2(M-1), 2(M-1)] Williamson symplectics
    kept: np.ndarray                # [M-1] rows per cut
    left_rows: np.ndarray           # [M-1] rows with res > err_tol
    timings: dict


def build_mps(sq_cov, d: int, chi: int, precision="split", out_dtype=torch.complex64, err_tol: float = 1e-10,
              device: int = 0, sites: Optional[List[int]] = None) -> MPS:
    dev = torch.device("cuda", device)
    sq = torch.as_tensor(sq_cov, dtype=torch.float64).to(dev).contiguous()
    M = sq.shape[0] // 2
    t = {}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res, num, S, kept_t = ops.cut_spectra(sq, d, chi, device=device)
    kept = kept_t.cpu().numpy()
    res_h = res.cpu().numpy()
    left_rows = np.array([int((res_h[c, : kept[c]] > err_tol).sum()) for c in range(M - 1)])
    lam = torch.where(res > err_tol, torch.sqrt(res.clamp_min(0)), torch.zeros_like(res))
    t["cuts_s"] = time.perf_counter() - t0
    Gammas = []
    t1 = time.perf_counter()
    for i in (range(M) if sites is None else sites):
        if i == 0:
            k0 = M - 1
            Sig, Z = ops.first_sigma(S[0, : 2 * k0, : 2 * k0].contiguous(), sq, device=device)
            kl = int(left_rows[0])
            G = ops.build_site(_lib.SITE_FIRST, Sig, num[0, :kl, :k0].contiguous(), lam[0, :kl].contiguous(), None, Z,
                               d, chi, precision, out_dtype, device)
        elif i == M - 1:
            Sig, Z = ops.site_sigma(None, S[M - 2, :2, :2].contiguous(), device=device)
            kr = int(kept[M - 2])
            G = ops.build_site(_lib.SITE_LAST, Sig, None, None, num[M - 2, :kr, :1].contiguous(), Z, d, chi,
                               precision, out_dtype, device)
        else:
            kl_modes = M - 1 - i
            kr_modes = M - i
            Sig, Z = ops.site_sigma(S[i, : 2 * kl_modes, : 2 * kl_modes].contiguous(),
                                    S[i - 1, : 2 * kr_modes, : 2 * kr_modes].contiguous(), device=device)
            kl = int(left_rows[i])
            kr = int(kept[i - 1])
            G = ops.build_site(_lib.SITE_MIDDLE, Sig, num[i, :kl, :kl_modes].contiguous(), lam[i, :kl].contiguous(),
                               num[i - 1, :kr, :kr_modes].contiguous(), Z, d, chi, precision, out_dtype, device)
        Gammas.append(G)
    torch.cuda.synchronize(dev)
    t["sites_s"] = time.perf_counter() - t1
    t["total_s"] = time.perf_counter() - t0
    return MPS(Gammas, lam, res, num, S, kept, left_rows, t)
