"""GPU parity of the per-cut truncation (kron_cpu.py:95-127) against the
reference's own res/num/S fixtures.  The GPU Williamson basis differs from
scipy's by a symplectic-orthogonal gauge per mode and orders modes by nu
descending, so labels are compared after mapping modes by nu."""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


def _omega(n):
    return np.block([[np.zeros((n, n)), np.eye(n)], [-np.eye(n), np.zeros((n, n))]])


def _ref_nu(sq_cov, L):
    M = sq_cov.shape[0] // 2
    sel = np.concatenate([np.arange(L, M), np.arange(L, M) + M])
    D, _ = R.williamson(sq_cov[np.ix_(sel, sel)])
    k = M - L
    return np.diag(D)[:k]


@pytest.mark.parametrize("fixture", ["tiny_M8.npz", "small_M16.npz"])
def test_cut_spectra_match_reference(cuda, golden, fixture):
    from bosonsupremacy_gb300 import ops
    t = golden(fixture)
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    sq = t["sq_cov"]
    res, num, S, kept = ops.cut_spectra(sq, d, chi)
    res, num, S, kept = res.cpu().numpy(), num.cpu().numpy(), S.cpu().numpy(), kept.cpu().numpy()
    for c in range(M - 1):
        L = c + 1
        k = M - L
        ref_res, ref_num = t[f"res_{c}"], t[f"num_{c}"].reshape(len(t[f"res_{c}"]), -1)
        assert kept[c] == len(ref_res), (c, kept[c], len(ref_res))
        got = res[c, : kept[c]]
        # Schmidt weights (Lambda^2): relative error per entry
        rel = np.abs(got - ref_res) / np.maximum(ref_res, 1e-300)
        big = ref_res > 1e-12
        assert rel[big].max() <= 1e-9, (c, rel[big].max())
        # Williamson symplectic: V = S D S^T and S Omega S^T = Omega
        sel = np.concatenate([np.arange(L, M), np.arange(L, M) + M])
        V = sq[np.ix_(sel, sel)]
        Sc = S[c, : 2 * k, : 2 * k]
        nu = _ref_nu(sq, L)
        mine_nu = np.sort(nu)[::-1]
        Dm = np.diag(np.concatenate([mine_nu, mine_nu]))
        assert np.abs(Sc @ Dm @ Sc.T - V).max() <= 1e-10 * np.abs(V).max(), c
        assert np.abs(Sc @ _omega(k) @ Sc.T - _omega(k)).max() <= 1e-10 * max(1.0, np.abs(Sc).max() ** 2), c
        # labels: reference columns reordered by nu descending (stable)
        perm = np.argsort(-nu, kind="stable")
        ref_lab = ref_num[:, perm]
        lab = num[c, : kept[c], :k]
        # rows whose weight is not tied with a neighbour must agree exactly
        untied = np.ones(len(ref_res), bool)
        gap = np.abs(np.diff(ref_res)) <= 1e-12 * ref_res[1:]
        untied[1:] &= ~gap
        untied[:-1] &= ~gap
        # modes with nu ~ 1 (vacuum) may be permuted among themselves; they hold 0 photons
        assert np.array_equal(lab[untied], ref_lab[untied]), c


def test_cut_spectra_rejects_non_pd(cuda):
    from bosonsupremacy_gb300 import ops
    from bosonsupremacy_gb300._lib import BSGError
    bad = -np.eye(8)
    with pytest.raises(BSGError, match="positive definite"):
        ops.cut_spectra(bad, 3, 8)


def test_cut_spectra_full_size_medium(cuda):
    """All 49 cuts of the M=50, d=6, chi=256 workload against the oracle
    (Schmidt weights per cut, and the photon count of every untied label)."""
    from bosonsupremacy_gb300 import ops, synthetic
    cfg = synthetic.MEDIUM
    _, sq = synthetic.lossy_covariances(cfg)
    res, num, S, kept = ops.cut_spectra(sq, cfg.d, cfg.chi)
    res, num, kept = res.cpu().numpy(), num.cpu().numpy(), kept.cpu().numpy()
    M = cfg.M
    for c in range(M - 1):
        # pruning to chi per step selects the same final set as max_dim=1e5 (see bsg_cuts.cu)
        ref_res, ref_num, _ = R.get_cumsum_kron(sq, c + 1, chi=cfg.chi, max_dim=cfg.chi, cutoff=cfg.d)
        assert kept[c] == len(ref_res), c
        got = res[c, : kept[c]]
        big = ref_res > 1e-12
        assert (np.abs(got - ref_res) / ref_res)[big].max() <= 1e-9, c
        untied = np.ones(len(ref_res), bool)
        gap = np.abs(np.diff(ref_res)) <= 1e-12 * ref_res[1:]
        untied[1:] &= ~gap
        untied[:-1] &= ~gap
        k = M - 1 - c
        assert np.array_equal(num[c, : kept[c], :k].sum(1)[untied], ref_num.reshape(len(ref_res), -1).sum(1)[untied])


def test_single_cut_entry_point(cuda, golden):
    """bsg_cut_spectrum (one cut, the reference's max_dim argument) equals
    the slab of that cut from bsg_cut_spectra, bit for bit; a max_dim below
    chi is rejected."""
    import torch
    from bosonsupremacy_gb300 import _lib, ops
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    res_all, num_all, S_all, kept_all = ops.cut_spectra(t["sq_cov"], d, chi)
    sq = torch.as_tensor(t["sq_cov"], dtype=torch.float64).cuda()
    h = _lib.Handle.get(0)
    lib = _lib.load()
    for L in (1, M // 2, M - 1):
        res = torch.empty(chi, dtype=torch.float64, device="cuda")
        num = torch.empty(chi, M - 1, dtype=torch.int8, device="cuda")
        S = torch.empty(2 * (M - 1), 2 * (M - 1), dtype=torch.float64, device="cuda")
        kept = torch.empty(1, dtype=torch.int32, device="cuda")
        _lib.check(lib.bsg_cut_spectrum(h.h, sq.data_ptr(), M, L, d, chi, 1e-12, 100000, res.data_ptr(),
                                        num.data_ptr(), S.data_ptr(), kept.data_ptr(), _lib.stream_ptr()),
                   "bsg_cut_spectrum")
        c = L - 1
        k = int(kept_all[c])
        assert int(kept.item()) == k
        assert torch.equal(res[:k], res_all[c, :k])
        assert torch.equal(num[:k], num_all[c, :k])
        n = 2 * (M - L)
        assert torch.equal(S[:n, :n], S_all[c, :n, :n])
    with pytest.raises(_lib.BSGError, match="max_dim"):
        _lib.check(lib.bsg_cut_spectrum(h.h, sq.data_ptr(), M, 1, d, chi, 1e-12, chi - 1, res.data_ptr(),
                                        num.data_ptr(), S.data_ptr(), kept.data_ptr(), _lib.stream_ptr()),
                   "bsg_cut_spectrum")
