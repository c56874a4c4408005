"""GPU parity of the transfer contraction (sampling_cpu.py:75-80 with fixed
photon numbers) against the oracle, on the reference's own Gamma/Lambda."""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


# sliced: ~42 bits of each operand row's scale (fixed point per row), so a
# probability 1e-6 of the largest keeps ~1e-10 relative
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 2e-5), ("split", 2e-5), ("sliced", 1e-9)])
def test_pattern_probabilities_on_reference_mps(cuda, golden, prec, tol):
    import torch
    from bosonsupremacy_gb300 import ops
    t = golden("tiny_M8.npz")
    M = int(t["M"])
    G = [torch.as_tensor(t[f"Gamma_{i}"]) for i in range(M)]
    L = np.stack([t[f"Lambda_{c}"] for c in range(M - 1)])
    pats = t["patterns"]
    amp = ops.pattern_amplitudes(G, L, pats, precision=prec).cpu().numpy()
    ref = R.pattern_amplitudes([t[f"Gamma_{i}"] for i in range(M)], list(L), pats)
    p, pr = np.abs(amp) ** 2, np.abs(ref) ** 2
    assert np.abs(p - t["pattern_probs"]).max() <= 1e-12 * pr.max() + tol * pr.max()
    big = pr > 1e-6 * pr.max()
    assert (np.abs(p[big] - pr[big]) / pr[big]).max() <= tol


def test_contraction_of_gpu_mps_medium_sample(cuda):
    """Random sample of <= 4-photon patterns of the M=50 workload: GPU
    contraction (fp64) of the GPU-built MPS vs the oracle contraction."""
    import torch
    from bosonsupremacy_gb300 import ops, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps
    cfg = synthetic.MEDIUM
    _, sq = synthetic.lossy_covariances(cfg)
    mps = build_mps(sq, cfg.d, cfg.chi, precision="split", out_dtype=torch.complex128)
    rng = np.random.default_rng(3)
    P = 400
    pats = np.zeros((P, cfg.M), np.int32)
    for p in range(P):
        k = rng.integers(0, 5)
        for _ in range(k):
            pats[p, rng.integers(0, cfg.M)] += 1
    pats = np.minimum(pats, cfg.d - 1)
    amp = ops.pattern_amplitudes(mps.Gammas, mps.Lambdas, pats, precision="fp64").cpu().numpy()
    G = [g.cpu().numpy() for g in mps.Gammas]
    Lam = mps.Lambdas.cpu().numpy()
    ref = R.pattern_amplitudes(G, list(Lam), pats)
    assert np.abs(amp - ref).max() <= 1e-10 * np.abs(ref).max()


def test_contract_patterns_alias(cuda, golden):
    """bsg_contract_patterns returns exactly bsg_pattern_amplitudes' result."""
    import ctypes
    import torch
    from bosonsupremacy_gb300 import _lib, ops
    t = golden("tiny_M8.npz")
    M, d = int(t["M"]), int(t["d"])
    G = [torch.as_tensor(t[f"Gamma_{i}"]).to(torch.complex128).cuda().contiguous() for i in range(M)]
    chi = G[0].shape[0]
    L = np.stack([t[f"Lambda_{c}"] for c in range(M - 1)]).astype(np.float64)
    want = ops.pattern_amplitudes(G, L, t["patterns"], precision="fp64")
    Lt = torch.as_tensor(L).cuda().contiguous()
    pats = torch.as_tensor(np.asarray(t["patterns"], np.int32)).cuda().contiguous()
    out = torch.empty(pats.shape[0], dtype=torch.complex128, device="cuda")
    ptrs = (ctypes.c_void_p * M)(*[g.data_ptr() for g in G])
    h = _lib.Handle.get(0)
    _lib.check(_lib.load().bsg_contract_patterns(h.h, ptrs, Lt.data_ptr(), M, chi, d, pats.data_ptr(),
                                                 pats.shape[0], _lib.PREC_FP64, out.data_ptr(), _lib.stream_ptr()),
               "bsg_contract_patterns")
    torch.cuda.synchronize()
    assert torch.equal(out, want.to(out.device))
