"""GPU parity of Sigma construction and the fused per-site Gamma build against
the reference's own outputs (tests/golden/tiny_M8.npz, produced by the
unmodified MPS_cpu.py in FP64)."""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


def _cuts(t):
    M = int(t["M"])
    return [(t[f"res_{c}"], t[f"num_{c}"], t[f"S_{c}"]) for c in range(M - 1)]


def _site_inputs(t, i, err_tol=1e-10):
    M = int(t["M"])
    cuts = _cuts(t)
    if i == 0:
        res, num, _ = cuts[0]
        keep = res > err_tol
        return num[keep].reshape(int(keep.sum()), -1), np.sqrt(res[keep]), None
    if i == M - 1:
        num_r = cuts[i - 1][1]
        return None, None, num_r.reshape(num_r.shape[0], -1)
    res, num, _ = cuts[i]
    keep = res > err_tol
    num_r = cuts[i - 1][1]
    return num[keep].reshape(int(keep.sum()), -1), np.sqrt(res[keep]), num_r.reshape(num_r.shape[0], -1)


def test_sigma_matches_reference(cuda, golden):
    from bosonsupremacy_gb300 import ops
    t = golden("tiny_M8.npz")
    M = int(t["M"])
    for i in range(M):
        if i == 0:
            Sig, Z = ops.first_sigma(t["S_0"], t["sq_cov"])
            blk = slice(0, M)
        elif i == M - 1:
            Sig, Z = ops.site_sigma(None, t[f"S_{M - 2}"])
            blk = slice(0, 2)
        else:
            Sig, Z = ops.site_sigma(t[f"S_{i}"], t[f"S_{i - 1}"])
            blk = slice(0, 2 * (M - i))
        ref = t[f"Sigma_{i}"]
        assert np.abs(Sig.cpu().numpy()[blk, blk] - ref[blk, blk]).max() < 1e-12, i
        assert abs(Z.item() - float(t[f"Z_{i}"])) < 1e-12 * float(t[f"Z_{i}"]), i


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-11), ("split", 1e-9), ("fp32", 1e-4)])
def test_gamma_matches_reference(cuda, golden, prec, tol):
    import torch
    from bosonsupremacy_gb300 import ops, _lib
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    for i in range(M):
        num_l, lam, num_r = _site_inputs(t, i)
        ref = t[f"Gamma_{i}"]
        Sig = t[f"Sigma_{i}"]
        Z = np.array([float(t[f"Z_{i}"])])
        kind = _lib.SITE_FIRST if i == 0 else _lib.SITE_LAST if i == M - 1 else _lib.SITE_MIDDLE
        G = ops.build_site(kind, Sig, num_l, lam, num_r, Z, d, chi, precision=prec,
                           out_dtype=torch.complex128).cpu().numpy()
        err = np.abs(G - ref).max() / np.abs(ref).max()
        assert err <= tol, (i, prec, err)
        assert np.all(G[ref == 0] == 0), i
