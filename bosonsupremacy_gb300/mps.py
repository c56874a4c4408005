"""Drop-in for MPS_cpu.py: per-site Gamma/Lambda on the GPU.

    python -m bosonsupremacy_gb300.mps --d D --chi CHI --dir ROOT/ [--precision split|fp64|fp32]

Same flags (MPS_cpu.py:7-15), same inputs -- ROOT/sq_cov.npy, ROOT/cov.npy and
the cut files ROOT/d_{D}_chi_{CHI}/{res,num,S}_i.npy written by kron_cpu.py or
by bosonsupremacy_gb300.kron -- and the same outputs: Gamma_i.npy complex64
[chi, chi, d] for i = 0..M-1 and Lambda_i.npy float32 [chi] for i = 0..M-2
(MPS_cpu.py:397-398, 523-525).  ``--fp64-out`` writes complex128/float64.

Function-level mirror of the reference's operator API (same names, argument
meaning and errors): ``hafnian(A)``, ``A_elem(Sigma, target, denominator,
max_memory_in_gb)``, ``get_target(num)``, ``push_to_end(array)``,
``get_Sigma_Z(S_l, S_r)`` (replaces get_U2_sq_U1 + get_Sigma),
``build_site(...)`` (one site) and ``build_sites(...)`` (a site range in one
pipelined call, what the script runs).  All arithmetic runs in libbsg; there
is no CPU path.
"""
from __future__ import annotations

import argparse
import time

import numpy as np
import torch

from . import _lib, dist, ops

ERR_TOL = 10 ** (-10)  # MPS_cpu.py:390


def hafnian(A, precision="fp64"):
    """Hafnians of a batch [B, n, n] (MPS_cpu.py:117-140)."""
    A = np.asarray(A)
    if A.ndim != 3 or A.shape[1] != A.shape[2]:
        raise ValueError("Matrix must be square")
    return ops.hafnian(A, precision=precision).cpu().numpy()


def A_elem(Sigma, target, denominator, max_memory_in_gb=0.5, precision="fp64"):
    """haf(Sigma[t][:, t]) / denominator with gather and hafnian times
    (MPS_cpu.py:334-355).  The gather is fused into the hafnian kernel, so the
    gather time is reported as 0 and the hafnian time covers both."""
    torch.cuda.synchronize()
    t0 = time.time()
    out = ops.hafnian_batched(Sigma, np.asarray(target, dtype=np.int32), np.asarray(denominator, dtype=np.float64),
                              precision=precision)
    torch.cuda.synchronize()
    return out.cpu().numpy(), time.time() - t0, 0.0


def get_target(num):
    """Expand Fock labels to repeated 1-based mode indices, left-aligned
    (MPS_cpu.py:314-332; host-side index bookkeeping as in the reference)."""
    num = np.asarray(num)
    rows, modes = num.shape
    width = int(num.sum(axis=1).max()) if rows else 0
    out = np.zeros((rows, width), dtype=np.int32)
    for r in range(rows):
        idx = np.repeat(np.arange(1, modes + 1, dtype=np.int32), num[r].astype(np.int64))
        out[r, : len(idx)] = idx
    return out


def push_to_end(array):
    """Right-align the non-zero entries of each row (MPS_cpu.py:39-47)."""
    out = np.zeros_like(array)
    for r in range(array.shape[0]):
        nz = array[r][array[r] != 0]
        if len(nz):
            out[r, -len(nz):] = nz
    return out


def get_Sigma_Z(S_l, S_r, sq_cov=None, device: int = 0):
    """Sigma and Z of a site from the Williamson symplectics of its two cuts
    (MPS_cpu.py:357-372 + 305-312 + 483).  Site 0 passes ``sq_cov`` (the pure
    covariance) instead of the full-state Williamson S (MPS_cpu.py:395)."""
    if sq_cov is not None:
        return ops.first_sigma(S_l, sq_cov, device=device)
    return ops.site_sigma(S_l, S_r, device=device)


def build_site(site, M, d, chi, sq_cov, path, precision="split", out_dtype=torch.complex64, err_tol=ERR_TOL,
               device: int = 0):
    """Gamma and Lambda of one site from the cut files in ``path``
    (the three branches of MPS_cpu.py:402-520)."""
    lam = np.zeros(chi, dtype=np.float64)
    if site == 0:
        res = np.load(path + "res_0.npy").astype(np.float64)
        num = np.load(path + "num_0.npy")
        S_l = np.load(path + "S_0.npy")
        keep = res > err_tol
        num = num[keep].reshape(int(keep.sum()), -1)
        res = res[keep]
        Sig, Z = get_Sigma_Z(S_l, None, sq_cov=sq_cov, device=device)
        lam[: len(res)] = np.sqrt(res)
        G = ops.build_site(_lib.SITE_FIRST, Sig, num, np.sqrt(res), None, Z, d, chi, precision, out_dtype,
                           device=device)
        return G, lam
    if site == M - 1:
        num_pre = np.load(path + f"num_{site - 1}.npy")
        num_pre = num_pre.reshape(num_pre.shape[0], -1)
        S_r = np.load(path + f"S_{site - 1}.npy")
        Sig, Z = get_Sigma_Z(None, S_r, device=device)
        G = ops.build_site(_lib.SITE_LAST, Sig, None, None, num_pre, Z, d, chi, precision, out_dtype, device=device)
        return G, None
    num_pre = np.load(path + f"num_{site - 1}.npy")
    num_pre = num_pre.reshape(num_pre.shape[0], -1)
    S_r = np.load(path + f"S_{site - 1}.npy")
    res = np.load(path + f"res_{site}.npy").astype(np.float64)
    num = np.load(path + f"num_{site}.npy")
    S_l = np.load(path + f"S_{site}.npy")
    keep = res > err_tol
    num = num[keep].reshape(int(keep.sum()), -1)
    res = res[keep]
    Sig, Z = get_Sigma_Z(S_l, S_r, device=device)
    lam[: len(res)] = np.sqrt(res)
    G = ops.build_site(_lib.SITE_MIDDLE, Sig, num, np.sqrt(res), num_pre, Z, d, chi, precision, out_dtype,
                       device=device)
    return G, lam


def load_cuts(path, M, chi, cuts, device: int = 0):
    """Device arrays of the given cuts' files (res_c, num_c, S_c as kron_cpu.py
    writes them; res may be float16 or float64) in bsg_cut_spectra's layout:
    res [M-1, chi] float64, num [M-1, chi, M-1] int8, S [M-1, 2(M-1), 2(M-1)]
    float64, kept [M-1] int32; the other cuts' rows stay zero."""
    nc = M - 1
    res = np.zeros((nc, chi))
    num = np.zeros((nc, chi, nc), dtype=np.int8)
    S = np.zeros((nc, 2 * nc, 2 * nc))
    kept = np.zeros(nc, dtype=np.int32)
    for c in cuts:
        r = np.load(path + f"res_{c}.npy").astype(np.float64)
        n_ = np.load(path + f"num_{c}.npy").reshape(len(r), -1)
        s_ = np.load(path + f"S_{c}.npy")
        k, m = len(r), nc - c
        if k > chi or n_.shape[1] != m or s_.shape != (2 * m, 2 * m):
            raise ValueError(f"cut {c}: files do not match M={M}, chi={chi}")
        res[c, :k] = r
        num[c, :k, :m] = n_
        S[c, : 2 * m, : 2 * m] = s_
        kept[c] = k
    dev = torch.device("cuda", device)
    return (torch.as_tensor(res).to(dev), torch.as_tensor(num).to(dev), torch.as_tensor(S).to(dev),
            torch.as_tensor(kept).to(dev))


def build_sites(s0, s1, M, d, chi, sq_cov, path, precision="split", out_dtype=torch.complex64, err_tol=ERR_TOL,
                device: int = 0):
    """Gamma of sites [s0, s1) and the Lambdas of the cuts they read, from the
    cut files in ``path``, in one pipelined library call (bsg_build_sites):
    Sigma of every site in one set of launches, one host wait, one DP launch
    set over all their items.  Returns (list of Gamma tensors, Lambdas
    [M-1, chi] float64 on the device)."""
    import ctypes
    dev = torch.device("cuda", device)
    cuts = range(max(0, s0 - 1), min(s1, M - 1))
    res, num, S, kept = load_cuts(path, M, chi, cuts, device)
    sq = torch.as_tensor(np.asarray(sq_cov, dtype=np.float64)).to(dev).contiguous()
    gam = [torch.empty(chi, chi, d, dtype=out_dtype, device=dev) for _ in range(s0, s1)]
    lam = torch.zeros(M - 1, chi, dtype=torch.float64, device=dev)
    odt = _lib.OUT_C128 if out_dtype == torch.complex128 else _lib.OUT_C64
    ptrs = (ctypes.c_void_p * len(gam))(*[g.data_ptr() for g in gam])
    h = _lib.Handle.get(device)
    _lib.check(_lib.load().bsg_build_sites(h.h, sq.data_ptr(), M, d, chi, float(err_tol), ops._prec(precision), odt,
                                           s0, s1, res.data_ptr(), num.data_ptr(), S.data_ptr(), kept.data_ptr(), ptrs,
                                           lam.data_ptr(), _lib.stream_ptr()),
               "bsg_build_sites")
    return gam, lam


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--d", type=int, help="Maximum number of photons per mode before displacement - 1.")
    p.add_argument("--chi", type=int, help="Bond dimension.")
    p.add_argument("--dir", type=str, help="Root directory.", default=0)
    p.add_argument("--precision", default="split", choices=["split", "fp64", "fp32"])
    p.add_argument("--fp64-out", action="store_true", help="write complex128 / float64")
    args = p.parse_args(argv)
    d, chi, rootdir = args.d, args.chi, args.dir
    path = rootdir + f"d_{d}_chi_{chi}/"
    sq_cov = np.load(rootdir + "sq_cov.npy")
    cov = np.load(rootdir + "cov.npy")
    M = len(cov) // 2
    gdt = torch.complex128 if args.fp64_out else torch.complex64
    ldt = "float64" if args.fp64_out else "float32"
    # under torchrun each rank writes the files of its own contiguous site range
    rank, world, local = dist.rank_world()
    device = local % max(1, torch.cuda.device_count())
    torch.cuda.set_device(device)
    s0, s1 = dist.shard_sites(M, world)[rank] if world > 1 else (0, M)
    t0 = time.time()
    gam, lam = build_sites(s0, s1, M, d, chi, sq_cov, path, args.precision, gdt, device=device)
    lam = lam.cpu().numpy()
    print(f"modes {s0}..{s1 - 1}: build {time.time() - t0:.4f} s")
    for site in range(s0, s1):
        np.save(path + f"Gamma_{site}.npy", gam[site - s0].cpu().numpy())
        if site < M - 1:
            np.save(path + f"Lambda_{site}.npy", lam[site].astype(ldt))


if __name__ == "__main__":
    main()
