"""Whole-build parity of the GPU path against the reference's own FP64 CPU
MPS on two of the five workloads (fixtures written by
tests/golden/make_golden_large.py, which runs the unmodified kron_cpu.py,
MPS_cpu.py and sampling_cpu.py FP64-promoted):

M=144, d=8, chi=1024 (Haar, r~U[1.2,1.6], eta=0.45) -- the headline workload:
  * Schmidt values Lambda of all 143 cuts against kron_cpu.py's weights:
    relative error <= 1e-8 per kept value (the near-degenerate middle cuts
    included), the same kept counts;
  * site 71 built by bsg_build_site from the reference's own cut files 70
    and 71 (same Williamson basis, so Gamma is comparable element-wise)
    against MPS_cpu.py's Gamma_71 on a stratified sample of its entries:
    1e-9 of max(|entry|, 1e-6 of the site's largest) for both DP
    arithmetics (both measure 1.9e-10: the difference between the
    reference's Bloch-Messiah Sigma and this build's Gauss-Jordan Sigma,
    not the DP's rounding).

M=50, d=6, chi=256 (Haar, r~U[0.8,1.2], eta=0.4) -- the whole build:
  * Lambda of all 49 cuts: relative error <= 1e-8;
  * probabilities of all 316 251 patterns with <= 4 photons, the GPU-built
    MPS (split and fp64 DP, complex128 Gamma) contracted on the GPU in FP64
    on the CUDA cores or by the sliced tensor-core path, against the
    reference MPS's: relative error <= 1e-6 for every pattern above 1e-8 of
    the largest probability.  With the reference's complex64
    Gamma storage the same comparison reaches only ~5e-5 (the rounding of
    Gamma alone, whatever the arithmetic), so that case is checked at 5e-4;
  * one- and two-point photon-number correlations of 10^5 samples drawn by
    the GPU sampler from the GPU-built MPS with the reference's random
    numbers (np.random.seed(2025), batches of 25 000, dd = d + 2, the
    reference's own sqrtW) against sampling_cpu.py's 10^5 samples from the
    reference MPS: the draws agree sample for sample except where a
    threshold falls within rounding of a cumulative probability, so
    |mean - mean_ref| and |cov - cov_ref| <= 2e-3 (about a third of one
    standard error of either estimate) and >= 99 % of the first 1024
    samples identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# ----------------------------------------------------------------- M=144
@pytest.fixture(scope="module")
def large(golden):
    return golden("large_M144.npz")


def _lambda_errors(res_gpu, kept_gpu, res_ref, kept_ref, site_tol=1e-10):
    """Per cut: max relative error of the kept Schmidt values sqrt(res)
    (sorted, so tied labels at the chi boundary compare by value)."""
    errs = []
    for c in range(len(kept_ref)):
        k = int(kept_ref[c])
        assert int(kept_gpu[c]) == k, (c, int(kept_gpu[c]), k)
        a = np.sort(res_gpu[c, :k])[::-1]
        b = np.sort(res_ref[c, :k])[::-1]
        big = b > site_tol
        la, lb = np.sqrt(a[big]), np.sqrt(b[big])
        errs.append(float((np.abs(la - lb) / lb).max()))
    return np.array(errs)


def test_large_lambda_matches_reference_all_cuts(cuda, large):
    import torch
    from bosonsupremacy_gb300.pipeline import build_mps
    M, d, chi = int(large["M"]), int(large["d"]), int(large["chi"])
    m = build_mps(large["sq_cov"], d, chi, precision="split")
    try:
        errs = _lambda_errors(m.res.cpu().numpy(), m.kept, large["res"], large["kept"])
    finally:
        del m
        torch.cuda.empty_cache()
    assert len(errs) == M - 1
    print(f"M=144 Lambda rel err per cut: max {errs.max():.3e} (cut {int(errs.argmax())}), "
          f"median {np.median(errs):.3e}; cuts 68-74: {np.array2string(errs[68:75], precision=2)}")
    assert errs.max() <= 1e-8, (int(errs.argmax()), errs.max())


@pytest.mark.parametrize("prec,tol", [("split", 1e-9), ("fp64", 1e-9)])
def test_large_site71_gamma_matches_reference(cuda, large, prec, tol):
    import torch
    from bosonsupremacy_gb300 import _lib, ops
    site = int(large["gamma_site"])
    d, chi = int(large["d"]), int(large["chi"])
    kept = large["kept"]
    res_l = large["res"][site, : kept[site]]
    num_l = large[f"num_{site}"]
    keep = res_l > 1e-10  # MPS_cpu.py:470-473
    num_l = num_l[keep].reshape(int(keep.sum()), -1)
    num_r = large[f"num_{site - 1}"]
    num_r = num_r.reshape(num_r.shape[0], -1)
    Sig, Z = ops.site_sigma(large[f"S_{site}"], large[f"S_{site - 1}"])
    G = ops.build_site(_lib.SITE_MIDDLE, Sig, num_l, np.sqrt(res_l[keep]), num_r, Z, d, chi, precision=prec,
                       out_dtype=torch.complex128)
    idx = torch.as_tensor(large["gamma_idx"].astype(np.int64), device=G.device)
    got = G[idx[:, 0], idx[:, 1], idx[:, 2]].cpu().numpy()
    nnz = int(torch.count_nonzero(G).item())
    del G
    ref = large["gamma_val"]
    scale = np.maximum(np.abs(ref), 1e-6 * float(large["gamma_absmax"]))
    err = np.abs(got - ref) / scale
    print(f"site {site} ({prec}): {len(ref)} entries, max rel err {err.max():.3e}")
    assert nnz == int(large["gamma_nonzero"])
    assert err.max() <= tol, err.max()


# ------------------------------------------------------------------ M=50
@pytest.fixture(scope="module")
def medium(golden):
    return golden("medium_M50.npz")


@pytest.fixture(scope="module")
def medium_builds(cuda, medium):
    import torch
    from bosonsupremacy_gb300.pipeline import build_mps
    d, chi = int(medium["d"]), int(medium["chi"])
    out = {p: build_mps(medium["sq_cov"], d, chi, precision=p, out_dtype=torch.complex128) for p in ("split", "fp64")}
    yield out
    del out
    torch.cuda.empty_cache()


@pytest.fixture(scope="module")
def medium_patterns(medium):
    from bosonsupremacy_gb300 import synthetic
    from oracle import reference_mps as R
    M, d = int(medium["M"]), int(medium["d"])
    pats = R.enumerate_patterns(M, 4, d)  # the fixture's pattern order
    assert len(pats) == int(medium["pattern_count"]) == len(synthetic.low_photon_patterns(M, 4, d))
    return pats, medium["pattern_prob_rel"].astype(np.float64) * float(medium["pattern_prob_max"])


@pytest.mark.parametrize("prec", ["split", "fp64"])
def test_medium_lambda_matches_reference(medium_builds, medium, prec):
    m = medium_builds[prec]
    errs = _lambda_errors(m.res.cpu().numpy(), m.kept, medium["res"], medium["kept"])
    assert errs.max() <= 1e-8, (int(errs.argmax()), errs.max())


def _prob_rel_err(p, pr, floor=1e-8):
    big = pr > floor * pr.max()
    return np.abs(p[big] - pr[big]) / pr[big]


@pytest.mark.parametrize("prec,contraction", [("split", "fp64"), ("fp64", "fp64"), ("split", "sliced")])
def test_medium_pattern_probabilities_match_reference(medium_builds, medium_patterns, prec, contraction):
    """The build (split or FP64 DP) contracted by the FP64 CUDA-core path or
    by the sliced tensor-core path (BF16 slice products, exact FP32
    accumulation, FP64 environments)."""
    from bosonsupremacy_gb300 import ops
    pats, pr = medium_patterns
    m = medium_builds[prec]
    amp = ops.pattern_amplitudes(m.Gammas, m.Lambdas, pats, precision=contraction)
    p = (amp.abs() ** 2).cpu().numpy()
    r = _prob_rel_err(p, pr)
    print(f"M=50 {prec} build, {contraction} contraction: {len(r)} patterns, prob rel err median "
          f"{np.median(r):.3e} max {r.max():.3e}")
    assert r.max() <= 1e-6, r.max()


def test_medium_probabilities_with_complex64_gamma(medium_builds, medium_patterns):
    """The reference's Gamma storage (complex64): its rounding alone limits
    the pattern probabilities to a few 1e-5; checked at 5e-4."""
    import torch
    from bosonsupremacy_gb300 import ops
    pats, pr = medium_patterns
    m = medium_builds["split"]
    g = [x.to(torch.complex64).to(torch.complex128) for x in m.Gammas]
    amp = ops.pattern_amplitudes(g, m.Lambdas, pats, precision="fp64")
    r = _prob_rel_err((amp.abs() ** 2).cpu().numpy(), pr)
    print(f"M=50 split build, complex64 Gamma: prob rel err median {np.median(r):.3e} max {r.max():.3e}")
    assert r.max() <= 5e-4, r.max()


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_medium_sampler_correlations_match_reference(medium_builds, medium, prec):
    import torch
    from bosonsupremacy_gb300 import sampling
    M, d = int(medium["M"]), int(medium["d"])
    m = medium_builds[prec]
    gam = m.Gammas if prec == "fp64" else [g.to(torch.complex64) for g in m.Gammas]
    N, batch, dd = int(medium["sample_n"]), int(medium["sample_batch"]), int(medium["sample_dd"])
    rng = np.random.RandomState(int(medium["sample_seed"]))
    s = np.concatenate([sampling.sample_mps(gam, m.Lambdas, medium["sqrtW"], dd, batch, rng, precision=prec)
                        for _ in range(0, N, batch)])
    assert s.shape == (N, M)
    same = (s[:1024] == medium["sample_head"]).all(axis=1).mean()
    s = s.astype(np.float64)
    dmean = np.abs(s.mean(0) - medium["sample_mean"]).max()
    dcov = np.abs(np.cov(s.T) - medium["sample_cov"]).max()
    print(f"M=50 sampler ({prec}): {same:.4f} of the first 1024 samples identical, |d mean| {dmean:.2e}, "
          f"|d cov| {dcov:.2e}")
    assert same >= 0.99, same
    assert dmean <= 2e-3, dmean
    assert dcov <= 2e-3, dcov
