"""The CPU baseline model (oracle/cpu_baseline.py, test and benchmark
infrastructure): its per-site group lists cover exactly the reference's
A_elem calls, its longest-first makespan spreads independent cuts / sites
over the cores, and its one-core and all-core estimates of the small 16-mode
workload agree in total work."""
import numpy as np
import pytest


def _small():
    from bosonsupremacy_gb300 import synthetic
    from oracle import reference_mps as R
    cfg = synthetic.NAMED["M16_d4_chi64"]
    _, sq = synthetic.lossy_covariances(cfg)
    cuts = [R.get_cumsum_kron(sq, c + 1, chi=cfg.chi, max_dim=cfg.chi, cutoff=cfg.d) for c in range(cfg.M - 1)]
    return cfg, sq, cuts


def test_site_groups_flatten_to_the_build_groups():
    from oracle import cpu_baseline
    cfg, _, cuts = _small()
    per_site = cpu_baseline.site_group_sizes(cuts, cfg.M, cfg.d)
    assert len(per_site) == cfg.M
    assert [g for s in per_site for g in s] == cpu_baseline.group_sizes(cuts, cfg.M, cfg.d)
    # every group is one A_elem call on a batch of >= 1 items (order 0: the
    # vacuum amplitude of site 0)
    assert all(n >= 0 and B >= 1 for s in per_site for n, B in s)


def test_makespan_longest_first():
    from oracle.cpu_baseline import _makespan
    # longest first: 5 -> a, 4 -> b, 3 -> b, 3 -> a, 3 -> b (the optimum, 9, is not sought)
    assert _makespan([5.0, 4.0, 3.0, 3.0, 3.0], 2) == pytest.approx(10.0)
    assert _makespan([1.0] * 8, 4) == pytest.approx(2.0)
    assert _makespan([10.0, 1.0, 1.0], 8) == pytest.approx(10.0)  # bounded by the largest task
    assert _makespan([2.0, 3.0], 1) == pytest.approx(5.0)


def test_all_core_estimate_of_the_small_workload():
    """Two sample processes (spawn): the build time is at most the one-core
    equivalent work and at least its share per core and the largest site."""
    from oracle import cpu_baseline
    cfg, sq, cuts = _small()
    e = cpu_baseline.estimate_full_build_parallel(sq, cfg.d, cfg.chi, cuts, procs=2, budget_s=1.0, timeout_s=300.0)
    assert e["procs"] == 2 and e["sites_per_s"] > 0
    assert e["build_s"] <= e["serial_s"] * (1 + 1e-12)
    assert e["build_s"] >= e["serial_s"] / 2 * (1 - 1e-12)
    assert e["build_s"] >= e["largest_site_s"]
    assert np.isclose(e["build_s"], e["kron_s"] + e["mps_s"])
