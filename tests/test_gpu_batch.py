"""The 64-instance uneven workload (M ~ U{8..48}, d ~ U{4..8}, chi in
{32, 64, 128, 256}, r ~ U[0.5, 1.4], eta ~ U[0.2, 0.6], each instance its
own Haar interferometer) built by bsg_build_mps_batch -- one launch per
phase over all instances, one DP launch set over the work items of every
site of every instance -- equals bsg_build_mps of each instance bit for bit
(every work item is evaluated by one lane with the same arithmetic
whichever bucket holds it)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,count", [("split", 64), ("fp64", 12)])
def test_batched_build_equals_looped(cuda, prec, count):
    import torch
    from bosonsupremacy_gb300 import synthetic
    from bosonsupremacy_gb300.pipeline import build_mps, build_mps_batch
    cfgs = synthetic.batch_configs(64)[:count]
    sqs = [synthetic.lossy_covariances(c)[1] for c in cfgs]
    batch = build_mps_batch(sqs, [c.d for c in cfgs], [c.chi for c in cfgs], precision=prec)
    assert len(batch) == count
    for cfg, sq, b in zip(cfgs, sqs, batch):
        a = build_mps(sq, cfg.d, cfg.chi, precision=prec)
        assert np.array_equal(a.kept, b.kept), cfg.name
        assert torch.equal(a.Lambdas, b.Lambdas), cfg.name
        assert torch.equal(a.res, b.res), cfg.name
        for i, (x, y) in enumerate(zip(a.Gammas, b.Gammas)):
            assert torch.equal(x, y), (cfg.name, i)
        del a
    del batch
    torch.cuda.empty_cache()


def test_batched_build_rejects_bad_instance(cuda):
    from bosonsupremacy_gb300 import _lib, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps_batch
    cfg = synthetic.batch_configs(64)[0]
    sq = synthetic.lossy_covariances(cfg)[1]
    with pytest.raises(_lib.BSGError):
        build_mps_batch([sq, sq], [cfg.d, cfg.chi + 1], [cfg.chi, cfg.chi])  # d > chi for instance 1


def test_batch_tuner_keeps_results(cuda):
    """autotune.tune_batch over a small grid of the DP's launch knobs picks a
    point of the grid, and the batched build after tuning gives the same
    Gammas as before (every knob only changes which warp runs an item)."""
    import torch
    from bosonsupremacy_gb300 import autotune, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps_batch
    cfgs = synthetic.batch_configs(64)[:8]
    sqs = [synthetic.lossy_covariances(c)[1] for c in cfgs]
    ds, chis = [c.d for c in cfgs], [c.chi for c in cfgs]
    before = build_mps_batch(sqs, ds, chis)
    saved = autotune.get_knobs()
    try:
        best, table = autotune.tune_batch(sqs, ds, chis, grid={"small_entries": (0, 64), "dp_quantum": (1, 8)}, reps=1)
        assert len(table) == 4 and tuple(best.values()) in table
        after = build_mps_batch(sqs, ds, chis)
    finally:
        autotune.set_knobs(**saved)
    for a, b in zip(before, after):
        for x, y in zip(a.Gammas, b.Gammas):
            assert torch.equal(x, y)
