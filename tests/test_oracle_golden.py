"""The oracle (CPU restatement of the reference) pinned against outputs of
the unmodified reference scripts (tests/golden/make_golden.py)."""
import numpy as np

from oracle import reference_mps as R


def test_hafnian_known_answers(golden):
    k = golden("hafnian_kat.npz")
    for n in [0, 1, 2, 3, 4, 5, 6, 8, 10, 12, 14]:
        assert np.array_equal(R.hafnian(k[f"A_{n}"]), k[f"haf_{n}"]), n


def test_a_elem_known_answers(golden):
    k = golden("hafnian_kat.npz")
    for n in [2, 4, 6, 8, 10]:
        amp, _, _ = R.A_elem(k["elem_Sigma"], k[f"elem_target_{n}"], k[f"elem_den_{n}"])
        assert np.array_equal(amp, k[f"elem_amp_{n}"]), n


def test_kron_and_mps_bit_exact(golden):
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    cuts = R.run_kron(t["sq_cov"], d, chi)
    for c in range(M - 1):
        assert np.array_equal(cuts[c][0], t[f"res_{c}"]), c
        assert np.array_equal(cuts[c][1], t[f"num_{c}"]), c
        assert np.array_equal(cuts[c][2], t[f"S_{c}"]), c
    mps = R.build_mps(t["sq_cov"], d, chi, cuts)
    for i in range(M):
        assert np.array_equal(mps[i][0], t[f"Gamma_{i}"]), i
        if i < M - 1:
            assert np.array_equal(mps[i][1], t[f"Lambda_{i}"]), i
    pats = t["patterns"]
    p = np.abs(R.pattern_amplitudes([mps[i][0] for i in range(M)], [mps[i][1] for i in range(M - 1)], pats)) ** 2
    assert np.allclose(p, t["pattern_probs"], rtol=1e-12, atol=0)


def test_small_config_spectra(golden):
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    for c in (0, 5, 14):
        res, num, S = R.get_cumsum_kron(t["sq_cov"], c + 1, chi=chi, cutoff=d)
        assert np.array_equal(res, t[f"res_{c}"]) and np.array_equal(num, t[f"num_{c}"]), c


def test_sampler_statistics_match_reference(golden):
    """Restated sampler (sampling_cpu.py:30-117) with the reference's seeded
    global RNG stream reproduces the reference's first samples exactly."""
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    G = [t[f"Gamma_{i}"] for i in range(M)]
    Lam = np.stack([t[f"Lambda_{c}"] for c in range(M - 1)], axis=1)
    thermal = t["cov"] - t["sq_cov"]
    thermal = thermal + 1.000001 * np.eye(len(thermal)) * np.abs(np.min(np.linalg.eigvalsh(thermal)))
    sqrtW = np.linalg.cholesky(thermal)
    rng = np.random.RandomState(int(t["sample_seed"]))
    s = R.sample(G, Lam, sqrtW, int(t["sample_dd"]), int(t["sample_n"]), rng)
    assert np.array_equal(s[:64], t["sample_head"])
    assert np.allclose(s.mean(0), t["sample_mean"])


def test_sampler_first_batch_of_1e5_matches_reference(golden):
    """Oracle MPS + restated sampler, first 25 000-sample batch of the
    reference's seeded 10^5-sample run on the M=16 instance: the first 256
    samples agree draw for draw."""
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    cuts = [(t[f"res_{c}"], t[f"num_{c}"], t[f"S_{c}"]) for c in range(M - 1)]
    mps = R.build_mps(t["sq_cov"], d, chi, cuts)
    G = [mps[i][0] for i in range(M)]
    Lam = np.stack([mps[c][1] for c in range(M - 1)], axis=1)
    thermal = t["cov"] - t["sq_cov"]
    thermal = thermal + 1.000001 * np.eye(len(thermal)) * np.abs(np.min(np.linalg.eigvalsh(thermal)))
    sqrtW = np.linalg.cholesky(thermal)
    rng = np.random.RandomState(int(t["big_sample_seed"]))
    s = R.sample(G, Lam, sqrtW, d + 2, int(t["big_sample_batch"]), rng)
    assert np.array_equal(s[:256], t["big_sample_head"])


def test_large_config_cut_spectra(golden):
    """The oracle's truncation to chi against kron_cpu.py on the M=144, d=8,
    chi=1024 workload (tests/golden/large_M144.npz): weights of the first,
    two middle and the last cut to 1e-10 relative (LAPACK's thread count
    moves the near-vacuum nu in their last bits, ~1e-11 in the weights),
    and the label rows of the two middle cuts
    the site-71 fixture was built from.  Rows of equal weight may come in
    another order (argsort ties, kron_cpu.py:113, 122), so the labels are
    compared as sets.  The Williamson symplectics differ by a rotation inside
    the near-degenerate (nu ~ 1) blocks, whose basis LAPACK leaves free, so
    S is checked for what fixes it: S Omega S^T = Omega and S^-1 V S^-T
    diagonal."""
    t = golden("large_M144.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    for c in (0, 70, 71, 142):
        res, num, S = R.get_cumsum_kron(t["sq_cov"], c + 1, chi=chi, cutoff=d)
        k = int(t["kept"][c])
        assert len(res) == k, c
        assert np.allclose(res, t["res"][c, :k], rtol=1e-10, atol=0), c  # LAPACK threading: ~1e-11
        if c in (70, 71):
            ref = t[f"num_{c}"]
            assert num.shape == ref.shape and set(map(bytes, num)) == set(map(bytes, ref)), c
            kk = M - c - 1
            sel = np.concatenate([np.arange(c + 1, M), np.arange(c + 1, M) + M])
            V = t["sq_cov"][np.ix_(sel, sel)]
            om = np.block([[np.zeros((kk, kk)), np.eye(kk)], [-np.eye(kk), np.zeros((kk, kk))]])
            for Sx in (S, t[f"S_{c}"]):
                assert np.abs(Sx @ om @ Sx.T - om).max() < 1e-9, c
                Si = -om @ Sx.T @ om
                D = Si @ V @ Si.T
                assert np.abs(D - np.diag(np.diag(D))).max() < 1e-9, c


def test_medium_config_cut_spectra(golden):
    """Same on the M=50, d=6, chi=256 workload (tests/golden/medium_M50.npz)."""
    t = golden("medium_M50.npz")
    d, chi = int(t["d"]), int(t["chi"])
    for c in (0, 24, 48):
        res, _, _ = R.get_cumsum_kron(t["sq_cov"], c + 1, chi=chi, cutoff=d)
        k = int(t["kept"][c])
        assert len(res) == k and np.allclose(res, t["res"][c, :k], rtol=1e-10, atol=0), c
