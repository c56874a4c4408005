"""DP launch knobs: range checks, and the launch split (small-table programs
in their own launch) leaves every Gamma bit-identical -- each item's DP runs
the same arithmetic whichever launch and scratch slice it lands in."""
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
                         (_lib.TUNE_DP_SMALL_BLOCKS, 0), (_lib.TUNE_DP_SCRATCH_MIB, 32), (99, 1)):
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
        for knobs in ({"small_entries": 0, "blocks_per_sm": 4},
                      {"small_entries": 16, "small_blocks": 2, "scratch_mib": 64},
                      {"small_entries": 4096, "small_blocks": 8}):
            autotune.set_knobs(**knobs)
            mps = build_mps(t["sq_cov"], d, chi, precision=prec, out_dtype=torch.complex128)
            outs.append([g.cpu().numpy() for g in mps.Gammas])
    finally:
        autotune.set_knobs(**saved)
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
