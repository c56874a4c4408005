"""DP launch knobs: range checks, and neither the launch split (small-table
programs in their own launch) nor yielding launches (warps leave after a
work quantum, blocks take table slots from a pool) change any Gamma bit --
each item's DP runs the same arithmetic whichever launch, warp and scratch
slice it lands in."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_knob_ranges(cuda):
    import ctypes as C
    from bosonsupremacy_gb300 import _lib, autotune
    lib = _lib.load()
    h = _lib.Handle.get(0)
    saved = autotune.get_knobs()
    try:
        for key, bad in ((_lib.TUNE_DP_BLOCKS_PER_SM, 0), (_lib.TUNE_DP_BLOCKS_PER_SM, 9),
                         (_lib.TUNE_DP_L1_CARVEOUT, 101), (_lib.TUNE_DP_SMALL_ENTRIES, -1),
                         (_lib.TUNE_DP_SMALL_BLOCKS, 0), (_lib.TUNE_DP_SCRATCH_MIB, 32),
                         (_lib.TUNE_DP_QUANTUM, -1), (99, 1)):
            assert lib.bsg_tune_set(h.h, key, bad) == -1, (key, bad)
        autotune.set_knobs(small_entries=128)
        assert autotune.get_knobs()["small_entries"] == 128
        v = C.c_int()
        assert lib.bsg_tune_get(h.h, 99, C.byref(v)) == -1
    finally:
        autotune.set_knobs(**saved)


@pytest.mark.parametrize("prec", ["split", "fp64"])
def test_launch_split_bit_identical(cuda, golden, prec):
    import torch
    from bosonsupremacy_gb300 import autotune
    from bosonsupremacy_gb300.pipeline import build_mps
    t = golden("small_M16.npz")
    d, chi = int(t["d"]), int(t["chi"])
    saved = autotune.get_knobs()
    outs = []
    try:
        for knobs in ({"small_entries": 0, "blocks_per_sm": 4, "dp_quantum": 0},
                      {"small_entries": 16, "small_blocks": 2, "scratch_mib": 64, "dp_quantum": 64},
                      {"small_entries": 4096, "small_blocks": 8, "dp_quantum": 1},
                      {"small_entries": 64, "small_blocks": 8, "dp_quantum": 1 << 20},
                      {"small_entries": 64, "small_blocks": 8, "dp_quantum": 2, "dp_hold": 1},
                      {"small_entries": 64, "small_blocks": 8, "dp_quantum": 2, "right_pct": 50, "left_pct": 20}):
            autotune.set_knobs(**knobs)
            mps = build_mps(t["sq_cov"], d, chi, precision=prec, out_dtype=torch.complex128)
            outs.append([g.cpu().numpy() for g in mps.Gammas])
    finally:
        autotune.set_knobs(**saved)
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


def test_fp64_helper_launch(cuda, golden):
    """Split build with the concurrent FP64 DP helper: items taken by the
    helper are computed in FP64, the rest in split precision; every Gamma
    agrees with the split-only build to split accuracy and the pattern
    probabilities still match the reference."""
    import torch
    from bosonsupremacy_gb300 import autotune
    from bosonsupremacy_gb300.pipeline import build_mps
    from oracle import reference_mps as R
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    saved = autotune.get_knobs()
    try:
        autotune.set_knobs(fp64_blocks=0)
        base = build_mps(t["sq_cov"], d, chi, precision="split", out_dtype=torch.complex128)
        autotune.set_knobs(fp64_blocks=2, blocks_per_sm=4, small_blocks=4)
        mps = build_mps(t["sq_cov"], d, chi, precision="split", out_dtype=torch.complex128)
    finally:
        autotune.set_knobs(**saved)
    for g0, g1 in zip(base.Gammas, mps.Gammas):
        a, b = g0.cpu().numpy(), g1.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-9 * max(1.0, np.abs(a).max())
    G = [g.cpu().numpy() for g in mps.Gammas]
    p = np.abs(R.pattern_amplitudes(G, list(mps.Lambdas.cpu().numpy()), t["patterns"])) ** 2
    pr = t["pattern_probs"]
    big = pr > 1e-8 * pr.max()
    assert (np.abs(p[big] - pr[big]) / pr[big]).max() <= 1e-6
