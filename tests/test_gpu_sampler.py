"""GPU sampler (sampling_cpu.py:30-117) and batched displacements
(sampling_cpu.py:133-148) against the oracle and the reference's own
samples.  The sampler takes the random numbers in the reference's draw order,
so a seeded numpy stream gives the reference's samples draw for draw; only a
threshold that falls within rounding of a cumulative probability can flip a
draw (and the rest of that sample's chain).

Tolerances:
  * displacements: |D - expm| <= 1e-12 (FP64, closed form vs scipy expm);
  * draw-for-draw: FP64 path reproduces the reference's stored samples
    exactly; split / FP32 paths differ in <= 0.5 % of sample rows;
  * one- and two-point correlations from 10^5 samples (M=16, GPU-built MPS
    and GPU sampler vs the reference's seeded 10^5-sample run):
    |mean_i - mean_i^ref| <= 2e-3 and |cov_ij - cov_ij^ref| <= 2e-3, about a
    third of one standard error of the 10^5-sample estimates.
"""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dd", [1, 4, 6, 10, 16])
def test_displacements_match_expm(cuda, dd):
    from bosonsupremacy_gb300 import ops
    rng = np.random.default_rng(dd)
    alpha = (rng.normal(size=(7, 5)) + 1j * rng.normal(size=(7, 5))) * 1.3
    alpha[0, 0] = 0.0
    D = ops.displacements(alpha, dd).cpu().numpy()
    ref = R.batch_displaces(dd, alpha)
    assert D.shape == ref.shape
    assert np.abs(D - ref).max() <= 1e-12


def _tiny(golden):
    from bosonsupremacy_gb300.sampling import thermal_sqrtW
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    G = [t[f"Gamma_{i}"] for i in range(M)]
    Lam = np.stack([t[f"Lambda_{c}"] for c in range(M - 1)])
    return t, M, d, chi, G, Lam, thermal_sqrtW(t["cov"], t["sq_cov"])


@pytest.mark.parametrize("prec", ["fp64", "split", "fp32"])
def test_sampler_reproduces_reference_samples(cuda, golden, prec):
    import torch
    from bosonsupremacy_gb300 import sampling
    t, M, d, chi, G, Lam, sqrtW = _tiny(golden)
    n, dd = int(t["sample_n"]), int(t["sample_dd"])
    Gd = [torch.as_tensor(g).cuda() for g in G]
    s = sampling.sample_mps(Gd, Lam, sqrtW, dd, n, np.random.RandomState(int(t["sample_seed"])), precision=prec)
    assert s.shape == (n, M) and s.dtype == np.int64
    # the oracle's samples for the same stream (pinned to the reference's head and mean)
    ref = R.sample(G, Lam.T, sqrtW, dd, n, np.random.RandomState(int(t["sample_seed"])))
    same = (s == ref).all(axis=1).mean()
    if prec == "fp64":
        assert np.array_equal(s[:64], t["sample_head"])
        assert same == 1.0
        assert np.allclose(s.mean(0), t["sample_mean"], rtol=0, atol=1e-12)
    else:
        assert same >= 0.995, same


def test_sampler_correlations_1e5(cuda, golden):
    """One- and two-point correlations of 10^5 samples drawn from the
    GPU-built MPS (split precision) by the GPU sampler (split precision)
    against the reference's 10^5 samples from its FP64 CPU MPS, same seed."""
    from bosonsupremacy_gb300 import sampling
    from bosonsupremacy_gb300.pipeline import build_mps
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    mps = build_mps(t["sq_cov"], d, chi, precision="split")
    sqrtW = sampling.thermal_sqrtW(t["cov"], t["sq_cov"])
    N, batch = int(t["big_sample_n"]), int(t["big_sample_batch"])
    rng = np.random.RandomState(int(t["big_sample_seed"]))
    s = np.concatenate([sampling.sample_mps(mps.Gammas, mps.Lambdas, sqrtW, d + 2, batch, rng, precision="split")
                        for _ in range(0, N, batch)]).astype(np.float64)
    assert s.shape == (N, M)
    assert (s[:256] == t["big_sample_head"]).all(axis=1).mean() >= 0.99
    dmean = np.abs(s.mean(0) - t["big_sample_mean"]).max()
    dcov = np.abs(np.cov(s.T) - t["big_sample_cov"]).max()
    assert dmean <= 2e-3, dmean
    assert dcov <= 2e-3, dcov


def test_sampler_cli_dropin(cuda, golden, tmp_path):
    """kron -> mps -> sampling CLIs on the same files the reference uses."""
    from bosonsupremacy_gb300 import kron, mps, sampling
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    root = str(tmp_path) + "/"
    np.save(root + "sq_cov.npy", t["sq_cov"])
    np.save(root + "cov.npy", t["cov"])
    args = ["--d", str(d), "--chi", str(chi), "--dir", root]
    kron.main(args)
    mps.main(args)
    np.random.seed(int(t["sample_seed"]))
    sampling.main(["--N", "3000", "--n", "1000", "--iter", "1", "--dd", str(d + 2)] + args)
    s = np.load(root + "samples_0.npy")
    assert s.shape == (3000, M) and s.dtype == np.int64
    assert s.min() >= 0 and s.max() <= d + 1
    # first batch = the reference's stream for n = 1000
    np.random.seed(int(t["sample_seed"]))
    G = [np.load(root + f"d_{d}_chi_{chi}/Gamma_{i}.npy") for i in range(M)]
    Lam = np.stack([np.load(root + f"d_{d}_chi_{chi}/Lambda_{c}.npy") for c in range(M - 1)], axis=1)
    ref = R.sample(G, Lam, sampling.thermal_sqrtW(t["cov"], t["sq_cov"]), d + 2, 1000, np.random)
    assert (s[:1000] == ref).all(axis=1).mean() >= 0.995


def test_sampler_rejects_bad_sizes(cuda, golden):
    import torch
    from bosonsupremacy_gb300 import _lib, ops
    t, M, d, chi, G, Lam, sqrtW = _tiny(golden)
    Gd = [torch.as_tensor(g).cuda() for g in G]
    z = np.zeros((2 * M, 4))
    u = np.zeros((M, 4))
    with pytest.raises(_lib.BSGError):
        ops.sample(Gd, Lam, sqrtW, z, u, d - 1, precision="fp64")  # dd < d
    with pytest.raises(_lib.BSGError):
        ops.sample(Gd, Lam, sqrtW, z, u, 17, precision="fp64")  # dd > 16
    with pytest.raises(_lib.BSGError):
        ops.displacements(np.zeros(3), 0)
