"""Size-independent properties of the whole-MPS build at the headline size
(M=144 modes, d=8, chi=1024 -- the reference's largest single-GPU workload,
9.7 GB of Gamma), where no CPU oracle finishes:

* the split-precision build agrees with the plain FP64 build: identical
  Schmidt values and cut labels (both run the same FP64 factorisations), and
  every Gamma entry within a few FP32 ulps (the two DP arithmetics differ by
  ~2^-44 relative before the complex64 rounding);
* the host-output build (every group's DP in four site parts, each part
  downloaded as it finishes) lands exactly the device build's Gammas and
  Lambdas;
* every Gamma is finite and not identically zero, every cut keeps at least
  one row, and the Schmidt weights of each cut are positive and sorted.

The largest banded workload (M=216, d=10, chi=2048) and instances of the
64-instance uneven workload get the same kind of checks.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORKLOAD = "M144_d8_chi1024"


@pytest.fixture(scope="module")
def full_builds(cuda):
    import torch
    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps
    cfg = synthetic.NAMED[WORKLOAD]
    _, sq = synthetic.lossy_covariances(cfg)
    split = build_mps(sq, cfg.d, cfg.chi, precision="split")
    fp64 = build_mps(sq, cfg.d, cfg.chi, precision="fp64")
    yield cfg, sq, split, fp64
    del split, fp64
    torch.cuda.empty_cache()


def test_split_matches_fp64_at_full_size(full_builds):
    import torch
    cfg, _, split, fp64 = full_builds
    assert np.array_equal(split.kept, fp64.kept)
    assert torch.equal(split.Lambdas, fp64.Lambdas)
    assert torch.equal(split.num, fp64.num)
    worst = 0.0
    for i, (a, b) in enumerate(zip(split.Gammas, fp64.Gammas)):
        scale = b.abs().max().item()
        assert scale > 0.0, i
        assert torch.isfinite(torch.view_as_real(a)).all(), i
        # elementwise: a few complex64 ulps of the entry, or of 1e-6 of the site's largest entry
        tol = 4.0 * 2.0 ** -23 * torch.maximum(b.abs(), torch.full_like(b.abs(), 1e-6 * scale))
        err = (a - b).abs()
        assert bool((err <= tol).all()), (i, (err / tol).max().item())
        worst = max(worst, (err.max() / scale).item())
    assert worst <= 1e-6


def test_cut_structure_at_full_size(full_builds):
    cfg, _, split, _ = full_builds
    res = split.res.cpu().numpy()
    for c in range(cfg.M - 1):
        k = int(split.kept[c])
        assert 1 <= k <= cfg.chi, c
        w = res[c, :k]
        assert (w > 0).all() and (np.diff(w) <= 0).all(), c
        assert w.sum() <= 1.0 + 1e-9, c


def test_host_output_build_matches_device_build_at_full_size(full_builds):
    import torch
    from bosonsupremacy_gb300.pipeline import build_mps_host
    cfg, sq, split, _ = full_builds
    M, d, chi = cfg.M, cfg.d, cfg.chi
    sqh = torch.as_tensor(sq).pin_memory()
    gh = [torch.empty(chi, chi, d, dtype=torch.complex64, pin_memory=True) for _ in range(M)]
    lh = torch.empty(M - 1, chi, dtype=torch.float64, pin_memory=True)
    build_mps_host(sqh, d, chi, gh, lh, precision="split")
    assert torch.equal(split.Lambdas.cpu(), lh)
    for i in range(M):
        assert torch.equal(split.Gammas[i], gh[i].to(split.Gammas[i].device, non_blocking=False)), i


def test_largest_banded_workload_properties(cuda, golden):
    """M=216, d=10, chi=2048, banded interferometer (72 GB of Gamma): the build
    completes, every Gamma is finite and non-zero, every cut keeps between 1
    and chi rows with positive, sorted weights summing to <= 1, and Lambda is
    the square root of the kept weights above the site tolerance.  The first
    32 cuts keep the reference's counts (FP64 kron_cpu.py,
    tests/golden/largest_M216.npz) and match its Schmidt values to 1e-8
    relative wherever the weight is above 1e-6, to 1e-4 down to 1e-10: the
    banded interferometer leaves modes with nbar ~1e-8 across these cuts,
    whose weights two FP64 methods determine only to ~1e-16 absolute in nu
    (the reference and an eigvalsh of the Hermitian form i Omega V disagree
    by up to 6e-6 on them, by 3e-10 above 1e-6)."""
    import torch
    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps
    cfg = synthetic.LARGEST
    ref = golden("largest_M216.npz")
    sq = ref["sq_cov"]
    m = build_mps(sq, cfg.d, cfg.chi, precision="split")
    try:
        for i, g in enumerate(m.Gammas):
            assert torch.isfinite(torch.view_as_real(g)).all(), i
            assert g.abs().max().item() > 0.0, i
        res = m.res.cpu().numpy()
        lam = m.Lambdas.cpu().numpy()
        for c in range(cfg.M - 1):
            k = int(m.kept[c])
            assert 1 <= k <= cfg.chi, c
            w = res[c, :k]
            assert (w > 0).all() and (np.diff(w) <= 0).all() and w.sum() <= 1.0 + 1e-9, c
            big = w > 1e-10
            assert np.allclose(lam[c, :k][big], np.sqrt(w[big]), rtol=1e-12, atol=0.0), c
        errs, errs_hi = [], []
        for c in range(len(ref["kept"])):
            k = int(ref["kept"][c])
            assert int(m.kept[c]) == k, (c, int(m.kept[c]), k)
            a, b = np.sort(res[c, :k])[::-1], ref["res"][c, :k]
            rel = np.abs(np.sqrt(a) - np.sqrt(b)) / np.sqrt(b)
            errs.append(float(rel[b > 1e-10].max()))
            errs_hi.append(float(rel[b > 1e-6].max()))
        print(f"M=216 first 32 cuts: Lambda rel err max {max(errs_hi):.3e} (weights > 1e-6), "
              f"{max(errs):.3e} (> 1e-10)")
        assert max(errs_hi) <= 1e-8, errs_hi
        assert max(errs) <= 1e-4, errs
    finally:
        del m
        torch.cuda.empty_cache()


@pytest.mark.parametrize("k", [0, 17, 42, 63])
def test_uneven_batch_instances_split_vs_fp64(cuda, k):
    """Instances of the 64-instance uneven workload (M 8-48, d 4-8, chi
    32-256): split and FP64 builds agree in Lambda exactly and in every Gamma
    entry to a few complex64 ulps."""
    import torch
    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps
    cfg = synthetic.batch_configs(64)[k]
    _, sq = synthetic.lossy_covariances(cfg)
    a = build_mps(sq, cfg.d, cfg.chi, precision="split")
    b = build_mps(sq, cfg.d, cfg.chi, precision="fp64")
    assert torch.equal(a.Lambdas, b.Lambdas)
    for i, (x, y) in enumerate(zip(a.Gammas, b.Gammas)):
        scale = y.abs().max().item()
        tol = 4.0 * 2.0 ** -23 * torch.maximum(y.abs(), torch.full_like(y.abs(), 1e-6 * scale))
        assert bool(((x - y).abs() <= tol).all()), (cfg.name, i)


@pytest.mark.parametrize("cut", [0, 1, 20, 47, 60, 65, 71, 76, 100, 141])
def test_williamson_symplectics_at_full_size(full_builds, cut):
    """Cut symplectics of the M=144 build (left cuts carry a vacuum cluster of
    up to 284 modes): S Omega S^T = Omega and S^-1 V S^-T = diag(nu, nu) with
    nu >= 1, V the sub-covariance of the cut's right block."""
    cfg, sq, split, _ = full_builds
    M = cfg.M
    L = cut + 1
    k = M - L
    sel = np.concatenate([np.arange(L, M), np.arange(L, M) + M])
    V = sq[np.ix_(sel, sel)]
    S = split.S[cut, : 2 * k, : 2 * k].cpu().numpy()
    om = np.block([[np.zeros((k, k)), np.eye(k)], [-np.eye(k), np.zeros((k, k))]])
    scale = max(1.0, np.abs(S).max() ** 2)
    sym_err = np.abs(S @ om @ S.T - om).max() / scale
    assert sym_err <= 1e-10, sym_err
    Si = -om @ S.T @ om  # the inverse of a symplectic matrix
    D = Si @ V @ Si.T
    dg = np.diag(D)
    nu = dg[:k]
    off = np.abs(D - np.diag(dg)) / np.sqrt(np.outer(np.abs(dg), np.abs(dg)))
    assert off.max() <= 1e-9, off.max()
    pair_err = np.abs(dg[k:] - nu).max() / nu.max()
    assert pair_err <= 1e-9, pair_err
    assert nu.min() >= 1.0 - 1e-9, nu.min()


@pytest.mark.parametrize("cut", [20, 31, 107, 160])
def test_williamson_restart_symplectics_M216(cuda, golden, cut):
    """Cuts of the banded M=216 workload whose refinement does not settle
    (near-vacuum modes ~1e-7 of the norm apart, mixed by the FP32 sweeps):
    they take the FP64 Jacobi restart from the FP32 sweeps' eigenvectors
    (cuts 20 and 31: the low-rank core; 107 and 160: the full matrix).  Their
    symplectics satisfy S Omega S^T = Omega and S^-1 V S^-T = diag(nu, nu)
    with nu >= 1 as the refined cuts of the M=144 build do."""
    from bosonsupremacy_gb300 import ops, synthetic
    cfg = synthetic.LARGEST
    sq = golden("largest_M216.npz")["sq_cov"]
    M = cfg.M
    L = cut + 1
    k = M - L
    _, _, S_all, _ = ops.cut_spectra(sq, cfg.d, cfg.chi, L0=L, n_cuts=1)
    S = S_all[0, : 2 * k, : 2 * k].cpu().numpy()
    sel = np.concatenate([np.arange(L, M), np.arange(L, M) + M])
    V = sq[np.ix_(sel, sel)]
    om = np.block([[np.zeros((k, k)), np.eye(k)], [-np.eye(k), np.zeros((k, k))]])
    scale = max(1.0, np.abs(S).max() ** 2)
    sym_err = np.abs(S @ om @ S.T - om).max() / scale
    assert sym_err <= 1e-10, sym_err
    Si = -om @ S.T @ om
    D = Si @ V @ Si.T
    dg = np.diag(D)
    nu = dg[:k]
    off = np.abs(D - np.diag(dg)) / np.sqrt(np.outer(np.abs(dg), np.abs(dg)))
    assert off.max() <= 1e-9, off.max()
    pair_err = np.abs(dg[k:] - nu).max() / nu.max()
    assert pair_err <= 1e-9, pair_err
    assert nu.min() >= 1.0 - 1e-9, nu.min()
