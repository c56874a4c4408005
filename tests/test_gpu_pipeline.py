"""End-to-end parity of the device-resident build (cut spectra -> Sigma ->
Gamma) against the reference's FP64 MPS through gauge-invariant outputs:
Lambda per cut and photon-number probabilities of every pattern with <= 4
photons (<= 3 for M > 16)."""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fixture", ["tiny_M8.npz", "small_M16.npz"])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_pattern_probabilities_match_reference(cuda, golden, fixture, prec):
    import torch
    from bosonsupremacy_gb300.pipeline import build_mps
    t = golden(fixture)
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    mps = build_mps(t["sq_cov"], d, chi, precision=prec, out_dtype=torch.complex128)
    G = [g.cpu().numpy() for g in mps.Gammas]
    Lam = mps.Lambdas.cpu().numpy()
    # Lambda per cut (relative, entries above 1e-6)
    for c in range(M - 1):
        ref = t[f"Lambda_{c}"]
        big = ref > 1e-6
        assert np.abs(Lam[c][big] - ref[big]).max() / ref[big].max() <= 1e-9, c
    pats = t["patterns"]
    p_ref = t["pattern_probs"]
    p = np.abs(R.pattern_amplitudes(G, list(Lam), pats)) ** 2
    big = p_ref > 1e-8 * p_ref.max()
    rel = np.abs(p[big] - p_ref[big]) / p_ref[big]
    assert rel.max() <= 1e-6, (prec, rel.max())
    assert np.abs(p - p_ref).max() <= 1e-9 * p_ref.max()


def test_build_to_host_matches_device_build(cuda, golden):
    """The host-output build (per-group downloads overlapping the build) lands
    exactly the device build's Gammas and Lambdas in pinned memory."""
    import torch
    from bosonsupremacy_gb300.pipeline import build_mps, build_mps_host
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    ref = build_mps(t["sq_cov"], d, chi, precision="split")
    sq = torch.as_tensor(t["sq_cov"]).pin_memory()
    gh = [torch.empty(chi, chi, d, dtype=torch.complex64, pin_memory=True) for _ in range(M)]
    lh = torch.empty(M - 1, chi, dtype=torch.float64, pin_memory=True)
    build_mps_host(sq, d, chi, gh, lh, precision="split")
    for a, b in zip(ref.Gammas, gh):
        assert torch.equal(a.cpu(), b)
    assert torch.equal(ref.Lambdas.cpu(), lh)
