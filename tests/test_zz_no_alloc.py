"""GPU test of bsg_site_sigma_noalloc, the allocation-free entry point for
callers that cannot call cudaMalloc (another allocator owns the device
memory, no implicit synchronisation allowed, or the host forbids raw device
allocation).  It is called through the C ABI and compared with the
allocating bsg_site_sigma on two calls in a row; this file is collected last
so that a run stopping at the first failure has run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, fn, S_l, S_r, handle=None):
    import torch
    from bosonsupremacy_gb300._lib import check
    Sr = torch.as_tensor(S_r, dtype=torch.float64).cuda().contiguous()
    Mr = Sr.shape[0] // 2
    Sl = torch.as_tensor(S_l, dtype=torch.float64).cuda().contiguous() if S_l is not None else None
    ml = Sl.shape[0] // 2 if Sl is not None else 0
    Sigma = torch.empty(2 * Mr, 2 * Mr, dtype=torch.complex128, device="cuda")
    Z = torch.empty(1, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sl = ctypes.c_void_p(Sl.data_ptr()) if Sl is not None else None
    if handle is None:
        check(fn(sl, ml, ctypes.c_void_p(Sr.data_ptr()), Mr, ctypes.c_void_p(Sigma.data_ptr()),
                 ctypes.c_void_p(Z.data_ptr()), st), "bsg_site_sigma_noalloc")
    else:
        check(fn(handle, sl, ml, ctypes.c_void_p(Sr.data_ptr()), Mr, ctypes.c_void_p(Sigma.data_ptr()),
                 ctypes.c_void_p(Z.data_ptr()), st), "bsg_site_sigma")
    torch.cuda.synchronize()
    return Sigma.cpu().numpy(), float(Z.item())


def test_noalloc_sigma_matches_allocating_entry_point(cuda, golden):
    from bosonsupremacy_gb300 import _lib
    lib = _lib.load()
    h = _lib.Handle.get(0)
    t = golden("tiny_M8.npz")
    M = int(t["M"])
    s = golden("small_M16.npz")
    cases = [(t["S_3"], t["S_2"]), (s["S_1"], s["S_0"]), (None, t[f"S_{M - 2}"])]
    for S_l, S_r in cases:  # consecutive calls share the scratch array
        got, Zg = _call(lib, lib.bsg_site_sigma_noalloc, S_l, S_r)
        ref, Zr = _call(lib, lib.bsg_site_sigma, S_l, S_r, handle=h.h)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        assert abs(Zg - Zr) <= 1e-12 * Zr


def test_noalloc_sigma_at_its_largest_size(cuda):
    """M_r = 160, the most modes the fixed scratch array holds: the two cuts
    next to site 1 of a synthetic 161-mode covariance (320 x 320 and
    318 x 318 Williamson symplectics), two calls in a row against
    bsg_site_sigma."""
    from bosonsupremacy_gb300 import _lib, ops, synthetic
    lib = _lib.load()
    h = _lib.Handle.get(0)
    cfg = synthetic.GBSConfig("M161_d4_chi8", 161, 4, 8, 0.5, 1.0, 0.4, seed=161)
    _, sq = synthetic.lossy_covariances(cfg)
    _, _, S, _ = ops.cut_spectra(sq, cfg.d, cfg.chi, L0=1, n_cuts=2)
    S = S.cpu().numpy()
    S_r, S_l = S[0, :320, :320], S[1, :318, :318]
    ref, Zr = _call(lib, lib.bsg_site_sigma, S_l, S_r, handle=h.h)
    for _ in range(2):
        got, Zg = _call(lib, lib.bsg_site_sigma_noalloc, S_l, S_r)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        assert abs(Zg - Zr) <= 1e-12 * Zr


def test_noalloc_sigma_rejects_oversize(cuda):
    import torch
    from bosonsupremacy_gb300 import _lib
    lib = _lib.load()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(x.data_ptr())
    rc = lib.bsg_site_sigma_noalloc(None, 0, p, 161, p, p, None)
    assert rc == -5
    assert b"160" in lib.bsg_last_error()
