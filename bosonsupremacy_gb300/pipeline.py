"""Full MPS construction on one GPU: cut spectra -> Sigma per site -> Gamma
per site, with every tensor resident in HBM.

Mirrors the two reference steps kron_cpu.py (all cuts) and MPS_cpu.py (all
sites) with the same outputs: Gamma_i [chi, chi, d] (complex64 by default,
as MPS_cpu.py:397) and Lambda_i [chi] = sqrt(res_i) of the rows with
res_i > err_tol, zero padded (MPS_cpu.py:398, 415, 484).
"""
from __future__ import annotations

import ctypes
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
              cut_tol: float = 1e-12, device: int = 0, out: Optional[List[torch.Tensor]] = None,
              handle: Optional[_lib.Handle] = None) -> MPS:
    """Whole MPS in one library call (bsg_build_mps).  ``out`` may supply the
    M Gamma tensors to fill (reused across calls); ``handle`` a library
    handle other than the device's shared one (its own program cache and
    scratch)."""
    dev = torch.device("cuda", device)
    sq = torch.as_tensor(sq_cov, dtype=torch.float64).to(dev).contiguous()
    M = sq.shape[0] // 2
    nc = M - 1
    if out is None:
        out = [torch.empty(chi, chi, d, dtype=out_dtype, device=dev) for _ in range(M)]
    odt = _lib.OUT_C128 if out[0].dtype == torch.complex128 else _lib.OUT_C64
    lam = torch.empty(nc, chi, dtype=torch.float64, device=dev)
    res = torch.empty(nc, chi, dtype=torch.float64, device=dev)
    num = torch.empty(nc, chi, M - 1, dtype=torch.int8, device=dev)
    S = torch.empty(nc, 2 * (M - 1), 2 * (M - 1), dtype=torch.float64, device=dev)
    kept = torch.empty(nc, dtype=torch.int32, device=dev)
    ptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in out])
    h = handle if handle is not None else _lib.Handle.get(device)
    t0 = time.perf_counter()
    _lib.check(_lib.load().bsg_build_mps(h.h, sq.data_ptr(), M, d, chi, float(cut_tol), float(err_tol),
                                         ops._prec(precision), odt, ptrs, lam.data_ptr(), res.data_ptr(),
                                         num.data_ptr(), S.data_ptr(), kept.data_ptr(), _lib.stream_ptr()),
               "bsg_build_mps")
    torch.cuda.synchronize(dev)
    t = {"total_s": time.perf_counter() - t0}
    kept_h = kept.cpu().numpy()
    res_h = res.cpu().numpy()
    left_rows = np.array([int((res_h[c, : kept_h[c]] > err_tol).sum()) for c in range(nc)])
    return MPS(out, lam, res, num, S, kept_h, left_rows, t)


def build_mps_batch(sq_covs, ds, chis, precision="split", out_dtype=torch.complex64, err_tol: float = 1e-10,
                    cut_tol: float = 1e-12, device: int = 0, outs: Optional[List[List[torch.Tensor]]] = None,
                    handle: Optional[_lib.Handle] = None) -> List[MPS]:
    """Independent instances (their own M, d, chi) in one library call
    (bsg_build_mps_batch): one launch per phase for all of them.  Returns
    one MPS per instance, equal to build_mps of that instance."""
    dev = torch.device("cuda", device)
    sqs = [torch.as_tensor(q, dtype=torch.float64).to(dev).contiguous() for q in sq_covs]
    n = len(sqs)
    Ms = [q.shape[0] // 2 for q in sqs]
    if outs is None:
        outs = [[torch.empty(c, c, d, dtype=out_dtype, device=dev) for _ in range(M)] for M, d, c in zip(Ms, ds, chis)]
    odt = _lib.OUT_C128 if outs[0][0].dtype == torch.complex128 else _lib.OUT_C64

    # every instance's cut outputs are views of one buffer per kind
    def views(dtype, shapes):
        sizes = [int(np.prod(sh)) for sh in shapes]
        flat = torch.empty(sum(sizes), dtype=dtype, device=dev)
        return [v.view(sh) for v, sh in zip(torch.split(flat, sizes), shapes)], flat

    lam, _ = views(torch.float64, [(M - 1, c) for M, c in zip(Ms, chis)])
    res, res_flat = views(torch.float64, [(M - 1, c) for M, c in zip(Ms, chis)])
    num, _ = views(torch.int8, [(M - 1, c, M - 1) for M, c in zip(Ms, chis)])
    S, _ = views(torch.float64, [(M - 1, 2 * (M - 1), 2 * (M - 1)) for M in Ms])
    kept, kept_flat = views(torch.int32, [(M - 1,) for M in Ms])

    def arr(ctype, xs):
        return (ctype * len(xs))(*xs)

    P = ctypes.c_void_p
    gptr = arr(P, [g.data_ptr() for o in outs for g in o])
    h = handle if handle is not None else _lib.Handle.get(device)
    t0 = time.perf_counter()
    _lib.check(_lib.load().bsg_build_mps_batch(
        h.h, n, arr(P, [q.data_ptr() for q in sqs]), arr(ctypes.c_int, Ms), arr(ctypes.c_int, list(ds)),
        arr(ctypes.c_int, list(chis)), float(cut_tol), float(err_tol), ops._prec(precision), odt, gptr,
        arr(P, [x.data_ptr() for x in lam]), arr(P, [x.data_ptr() for x in res]), arr(P, [x.data_ptr() for x in num]),
        arr(P, [x.data_ptr() for x in S]), arr(P, [x.data_ptr() for x in kept]), _lib.stream_ptr()),
        "bsg_build_mps_batch")
    kept_all = kept_flat.cpu().numpy()
    res_all = res_flat.cpu().numpy()
    t = {"total_s": time.perf_counter() - t0}
    out = []
    k0 = r0 = 0
    for i in range(n):
        nc, c = Ms[i] - 1, chis[i]
        kh = kept_all[k0:k0 + nc]
        rh = res_all[r0:r0 + nc * c].reshape(nc, c)
        k0, r0 = k0 + nc, r0 + nc * c
        left = ((rh > err_tol) & (np.arange(c)[None, :] < kh[:, None])).sum(axis=1)
        out.append(MPS(outs[i], lam[i], res[i], num[i], S[i], kh, left, t))
    return out


def build_mps_host(sq_cov_host: torch.Tensor, d: int, chi: int, gammas_host: List[torch.Tensor],
                   lambdas_host: torch.Tensor, precision="split", device: int = 0,
                   device_out: Optional[List[torch.Tensor]] = None, err_tol: float = 1e-10,
                   cut_tol: float = 1e-12) -> None:
    """Host-buffer form of build_mps: the covariance is copied in from (pinned)
    host memory and every Gamma_i and the Lambdas land in the given pinned
    host tensors; each build group's Gammas are downloaded while the other
    groups are still computing (bsg_build_mps_to_host)."""
    dev = torch.device("cuda", device)
    sq = sq_cov_host.to(dev, non_blocking=True)
    M = sq.shape[0] // 2
    nc = M - 1
    out = device_out
    if out is None:
        out = [torch.empty(chi, chi, d, dtype=gammas_host[0].dtype, device=dev) for _ in range(M)]
    if any(not g.is_pinned() for g in gammas_host) or not lambdas_host.is_pinned():
        raise ValueError("build_mps_host: host outputs must be pinned")
    odt = _lib.OUT_C128 if out[0].dtype == torch.complex128 else _lib.OUT_C64
    lam = torch.empty(nc, chi, dtype=torch.float64, device=dev)
    res = torch.empty(nc, chi, dtype=torch.float64, device=dev)
    num = torch.empty(nc, chi, M - 1, dtype=torch.int8, device=dev)
    S = torch.empty(nc, 2 * (M - 1), 2 * (M - 1), dtype=torch.float64, device=dev)
    kept = torch.empty(nc, dtype=torch.int32, device=dev)
    dptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in out])
    hptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in gammas_host])
    h = _lib.Handle.get(device)
    _lib.check(_lib.load().bsg_build_mps_to_host(h.h, sq.data_ptr(), M, d, chi, float(cut_tol), float(err_tol),
                                                 ops._prec(precision), odt, dptrs, hptrs, lam.data_ptr(),
                                                 lambdas_host.data_ptr(), res.data_ptr(), num.data_ptr(),
                                                 S.data_ptr(), kept.data_ptr(), _lib.stream_ptr()),
               "bsg_build_mps_to_host")
