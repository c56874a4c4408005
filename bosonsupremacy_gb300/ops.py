"""Device-side operators of the MPS construction (thin wrappers over libbsg).

Every function takes and returns torch CUDA tensors; torch only supplies the
device buffers and the current stream.  All arithmetic runs in libbsg's
sm_103a kernels.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import torch

from . import _lib
from ._lib import Handle, check, ptr, stream_ptr

C128 = torch.complex128


def _prec(precision) -> int:
    if isinstance(precision, int):
        return precision
    return _lib.PRECISIONS[precision]


def _dev(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(x, dtype=dtype, device=device).contiguous()


def hafnian_batched(Sigma, targets, denominator=None, precision="fp64", device: int = 0) -> torch.Tensor:
    """out[b] = haf(Sigma[t_b][:, t_b]) / denominator[b]  (the A_elem seam,
    MPS_cpu.py:334-355).  Sigma [n_len, n_len] complex, targets [B, n] int."""
    dev = torch.device("cuda", device)
    Sig = _dev(Sigma, C128, dev)
    tgt = _dev(targets, torch.int32, dev)
    if tgt.dim() != 2:
        raise ValueError("targets must be [B, n]")
    B, n = tgt.shape
    den = None if denominator is None else _dev(denominator, torch.float64, dev)
    out = torch.empty(B, dtype=C128, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_hafnian_batched(h.h, ptr(Sig), Sig.shape[0], ptr(tgt) if B * n else None, n, B, ptr(den),
                                          _prec(precision), ptr(out), stream_ptr()), "bsg_hafnian_batched")
    return out


def hafnian(A, precision="fp64", device: int = 0) -> torch.Tensor:
    """Hafnians of a batch [B, n, n] of symmetric matrices (MPS_cpu.py:117-140)."""
    dev = torch.device("cuda", device)
    At = _dev(A, C128, dev)
    B, n, _ = At.shape
    out = torch.empty(B, dtype=C128, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_hafnian_matrices(h.h, ptr(At), n, B, _prec(precision), ptr(out), stream_ptr()),
          "bsg_hafnian_matrices")
    return out


def site_sigma(S_l, S_r, device: int = 0) -> Tuple[torch.Tensor, torch.Tensor]:
    """Sigma and Z of a middle or last site from the Williamson symplectics of
    cuts site (S_l, empty for the last site) and site-1 (S_r)."""
    dev = torch.device("cuda", device)
    Sr = _dev(S_r, torch.float64, dev)
    Mr = Sr.shape[0] // 2
    Sl = None
    ml = 0
    if S_l is not None and (S_l.numel() if isinstance(S_l, torch.Tensor) else len(S_l)) > 0:
        Sl = _dev(S_l, torch.float64, dev)
        ml = Sl.shape[0] // 2
    Sigma = torch.empty(2 * Mr, 2 * Mr, dtype=C128, device=dev)
    Z = torch.empty(1, dtype=torch.float64, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_site_sigma(h.h, ptr(Sl), ml, ptr(Sr), Mr, ptr(Sigma), ptr(Z), stream_ptr()),
          "bsg_site_sigma")
    return Sigma, Z


def first_sigma(S_0, sq_cov, device: int = 0) -> Tuple[torch.Tensor, torch.Tensor]:
    """Sigma (output block) and Z of site 0 from cut 0's symplectic and the pure covariance."""
    dev = torch.device("cuda", device)
    sq = _dev(sq_cov, torch.float64, dev)
    M = sq.shape[0] // 2
    S0 = _dev(S_0, torch.float64, dev) if M > 1 else None
    Sigma = torch.empty(2 * M, 2 * M, dtype=C128, device=dev)
    Z = torch.empty(1, dtype=torch.float64, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_first_sigma(h.h, ptr(S0), M, ptr(sq), ptr(Sigma), ptr(Z), stream_ptr()),
          "bsg_first_sigma")
    return Sigma, Z


def build_site(kind: int, Sigma, num_l, lambda_l, num_r, Z, d: int, chi: int, precision="fp64",
               out_dtype=torch.complex64, device: int = 0, out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Gamma [chi, chi, d] of one site (MPS_cpu.py:402-520).  ``num_l`` are the
    kept labels of cut ``site`` (rows with res > err_tol), ``num_r`` all labels
    of cut ``site-1``; ``lambda_l`` = sqrt(res) of the kept rows."""
    dev = torch.device("cuda", device)
    Sig = _dev(Sigma, C128, dev)
    Mr = Sig.shape[0] // 2
    if kind != _lib.SITE_LAST:
        nl = _dev(num_l, torch.int8, dev).reshape(len(num_l), -1).contiguous()
        kl, ml = nl.shape
        lam = _dev(lambda_l, torch.float64, dev)
    else:
        nl, kl, ml, lam = None, 0, 0, None
    if kind != _lib.SITE_FIRST:
        nr = _dev(num_r, torch.int8, dev).reshape(len(num_r), -1).contiguous()
        kr, mr = nr.shape
    else:
        nr, kr, mr = None, 0, 0
    Zt = _dev(Z, torch.float64, dev).reshape(-1)
    if out is None:
        out = torch.empty(chi, chi, d, dtype=out_dtype, device=dev)
    odt = _lib.OUT_C128 if out.dtype == torch.complex128 else _lib.OUT_C64
    h = Handle.get(device)
    check(_lib.load().bsg_build_site(h.h, kind, ptr(Sig), Mr, ptr(nl) if kl * ml else None, kl, ml, ptr(lam),
                                     ptr(nr) if kr * mr else None, kr, mr, ptr(Zt), d, chi, _prec(precision), odt,
                                     ptr(out), stream_ptr()), "bsg_build_site")
    return out


def cut_spectra(sq_cov, d: int, chi: int, L0: int = 1, n_cuts: Optional[int] = None, err_tol: float = 1e-12,
                device: int = 0):
    """Schmidt weights, Fock labels and Williamson symplectics of cuts
    L0 .. L0+n_cuts-1 (kron_cpu.py:95-127 for each).  Returns device tensors
    res [n, chi] f64, num [n, chi, M-1] int8, S [n, 2(M-1), 2(M-1)] f64 and
    kept [n] int32; cut c uses the leading (M-L) label columns and the
    leading 2(M-L) block of S."""
    dev = torch.device("cuda", device)
    sq = _dev(sq_cov, torch.float64, dev)
    M = sq.shape[0] // 2
    if n_cuts is None:
        n_cuts = M - L0
    res = torch.empty(n_cuts, chi, dtype=torch.float64, device=dev)
    num = torch.empty(n_cuts, chi, M - 1, dtype=torch.int8, device=dev)
    S = torch.empty(n_cuts, 2 * (M - 1), 2 * (M - 1), dtype=torch.float64, device=dev)
    kept = torch.empty(n_cuts, dtype=torch.int32, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_cut_spectra(h.h, ptr(sq), M, L0, n_cuts, d, chi, float(err_tol), ptr(res), ptr(num),
                                      ptr(S), ptr(kept), stream_ptr()), "bsg_cut_spectra")
    return res, num, S, kept


def pattern_amplitudes(Gammas: Sequence[torch.Tensor], Lambdas, patterns, precision="fp64", device: int = 0):
    """Amplitudes of photon patterns [P, M] of the MPS (sampling_cpu.py:75-80
    with fixed photon numbers).  Gammas: M device tensors [chi, chi, d]
    (complex128 for fp64 and sliced, complex64 otherwise); Lambdas [M-1, chi]."""
    import ctypes
    dev = torch.device("cuda", device)
    M = len(Gammas)
    chi, _, d = Gammas[0].shape
    want = C128 if _prec(precision) in (_lib.PREC_FP64, _lib.PREC_SLICED) else torch.complex64
    G = [g.to(device=dev, dtype=want).contiguous() for g in Gammas]
    lam = _dev(Lambdas, torch.float64, dev)
    pat = _dev(patterns, torch.int32, dev)
    P = pat.shape[0]
    amp = torch.empty(P, dtype=C128, device=dev)
    ptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in G])
    h = Handle.get(device)
    check(_lib.load().bsg_pattern_amplitudes(h.h, ptrs, ptr(lam), M, chi, d, ptr(pat), P, _prec(precision), ptr(amp),
                                             stream_ptr()), "bsg_pattern_amplitudes")
    return amp


def gemm_sliced(A, B, device: int = 0) -> torch.Tensor:
    """C = A B^T in FP64 from BF16 fixed-point slice products on the tensor
    cores (bsg_gemm_sliced); A [M, K], B [N, K] float64, K % 8 == 0."""
    dev = torch.device("cuda", device)
    At = _dev(A, torch.float64, dev)
    Bt = _dev(B, torch.float64, dev)
    M, K = At.shape
    N = Bt.shape[0]
    C = torch.empty(M, N, dtype=torch.float64, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_gemm_sliced(h.h, ptr(At), ptr(Bt), ptr(C), M, N, K, stream_ptr()), "bsg_gemm_sliced")
    return C


def displacements(alpha, dd: int, device: int = 0) -> torch.Tensor:
    """D(alpha) = expm(alpha a^dag - alpha^* a) in dd dimensions for every
    entry of `alpha` (sampling_cpu.py:133-148): complex128 [..., dd, dd]."""
    dev = torch.device("cuda", device)
    a = _dev(alpha, C128, dev)
    out = torch.empty(*a.shape, dd, dd, dtype=C128, device=dev)
    h = Handle.get(device)
    check(_lib.load().bsg_displacements(h.h, ptr(a), a.numel(), int(dd), ptr(out), stream_ptr()), "bsg_displacements")
    return out


def sample(Gammas: Sequence[torch.Tensor], Lambdas, sqrtW, normals, uniforms, dd: int, precision="split",
           device: int = 0) -> torch.Tensor:
    """Photon-number samples [n, M] int64 (sampling_cpu.py:30-117) for the
    given random numbers: normals [2M, n] and per-site thresholds [M, n]."""
    import ctypes
    dev = torch.device("cuda", device)
    M = len(Gammas)
    chi, _, d = Gammas[0].shape
    want = C128 if _prec(precision) == _lib.PREC_FP64 else torch.complex64
    G = [g.to(device=dev, dtype=want).contiguous() for g in Gammas]
    lam = _dev(Lambdas, torch.float64, dev)
    W = _dev(sqrtW, torch.float64, dev)
    z = _dev(normals, torch.float64, dev)
    u = _dev(uniforms, torch.float64, dev)
    n = z.shape[1]
    if tuple(lam.shape) != (M - 1, chi) or tuple(W.shape) != (2 * M, 2 * M) or tuple(u.shape) != (M, n):
        raise ValueError("sample: expected Lambdas [M-1, chi], sqrtW [2M, 2M], normals [2M, n], uniforms [M, n]")
    out = torch.empty(n, M, dtype=torch.int64, device=dev)
    ptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in G])
    h = Handle.get(device)
    check(_lib.load().bsg_sample(h.h, ptrs, ptr(lam), M, chi, d, int(dd), ptr(W), ptr(z), ptr(u), n, _prec(precision),
                                 ptr(out), stream_ptr()), "bsg_sample")
    return out
