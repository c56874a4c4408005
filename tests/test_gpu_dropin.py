"""The drop-in CLIs (kron_cpu.py / MPS_cpu.py contracts) on the GPU, and
interoperability with the reference's own files in both directions."""
import os

import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu


def _write_inputs(t, root):
    np.save(os.path.join(root, "sq_cov.npy"), t["sq_cov"])
    np.save(os.path.join(root, "cov.npy"), t["cov"])


def test_cli_pipeline_matches_reference(cuda, golden, tmp_path):
    from bosonsupremacy_gb300 import kron, mps
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    root = str(tmp_path) + "/"
    _write_inputs(t, root)
    args = ["--d", str(d), "--chi", str(chi), "--dir", root]
    kron.main(args)
    mps.main(args + ["--precision", "split", "--fp64-out"])
    path = root + f"d_{d}_chi_{chi}/"
    G = [np.load(path + f"Gamma_{i}.npy") for i in range(M)]
    L = [np.load(path + f"Lambda_{i}.npy") for i in range(M - 1)]
    assert G[0].shape == (chi, chi, d) and G[0].dtype == np.complex128
    for c in range(M - 1):
        ref = t[f"Lambda_{c}"]
        big = ref > 1e-6
        assert np.abs(L[c][big] - ref[big]).max() <= 1e-9 * ref.max()
    p = np.abs(R.pattern_amplitudes(G, L, t["patterns"])) ** 2
    pr = t["pattern_probs"]
    big = pr > 1e-8 * pr.max()
    assert (np.abs(p[big] - pr[big]) / pr[big]).max() <= 1e-6


def test_reference_cut_files_give_reference_gamma(cuda, golden, tmp_path):
    """Our MPS step on the reference's own kron output reproduces the
    reference's Gamma element-wise (same Williamson basis, same gauge)."""
    from bosonsupremacy_gb300 import mps
    t = golden("tiny_M8.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    root = str(tmp_path) + "/"
    _write_inputs(t, root)
    path = root + f"d_{d}_chi_{chi}/"
    os.makedirs(path)
    for c in range(M - 1):
        np.save(path + f"res_{c}.npy", t[f"res_{c}"])
        np.save(path + f"num_{c}.npy", t[f"num_{c}"])
        np.save(path + f"S_{c}.npy", t[f"S_{c}"])
    mps.main(["--d", str(d), "--chi", str(chi), "--dir", root, "--precision", "fp64", "--fp64-out"])
    for i in range(1, M):  # site 0 uses the pure covariance: gauge of its input side differs by design
        G = np.load(path + f"Gamma_{i}.npy")
        ref = t[f"Gamma_{i}"]
        assert np.abs(G - ref).max() <= 1e-11 * np.abs(ref).max(), i
    G0 = np.load(path + "Gamma_0.npy")
    assert np.abs(G0 - t["Gamma_0"]).max() <= 1e-11 * np.abs(t["Gamma_0"]).max()


def test_oracle_on_our_cut_files_matches_our_gamma(cuda, golden, tmp_path):
    """The reference algorithm (oracle) run on OUR kron output gives our Gamma."""
    from bosonsupremacy_gb300 import kron, mps
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    root = str(tmp_path) + "/"
    _write_inputs(t, root)
    args = ["--d", str(d), "--chi", str(chi), "--dir", root]
    kron.main(args)
    path = root + f"d_{d}_chi_{chi}/"
    cuts = [(np.load(path + f"res_{c}.npy"), np.load(path + f"num_{c}.npy"), np.load(path + f"S_{c}.npy"))
            for c in range(M - 1)]
    for site in (1, 7, M - 1):
        G, _ = mps.build_site(site, M, d, chi, t["sq_cov"], path, precision="split",
                              out_dtype=__import__("torch").complex128)
        G = G.cpu().numpy()
        G_ref, _ = R.build_site(site, M, d, chi, t["sq_cov"], cuts)
        assert np.abs(G - G_ref).max() <= 1e-9 * np.abs(G_ref).max(), site


def test_cli_steps_sharded_over_ranks(cuda, golden, tmp_path):
    """Both CLI steps under a torchrun-style environment with two ranks (run
    one after the other here, on the one GPU): every rank writes the files of
    its own cut / site range, and together they are the single-rank files."""
    import subprocess
    import sys
    t = golden("small_M16.npz")
    M, d, chi = int(t["M"]), int(t["d"]), int(t["chi"])
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = {}
    for world in (1, 2):
        root = str(tmp_path / f"w{world}") + "/"
        os.makedirs(root)
        _write_inputs(t, root)
        args = ["--d", str(d), "--chi", str(chi), "--dir", root]
        for step in ("kron", "mps"):
            for rank in range(world):
                env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK="0")
                r = subprocess.run([sys.executable, "-m", f"bosonsupremacy_gb300.{step}"] + args,
                                   cwd=repo, env=env, capture_output=True, text=True, timeout=600)
                assert r.returncode == 0, r.stderr[-2000:]
        path = root + f"d_{d}_chi_{chi}/"
        outs[world] = {name: np.load(path + name) for name in sorted(os.listdir(path)) if name.endswith(".npy")}
    assert outs[1].keys() == outs[2].keys()
    assert len([n for n in outs[1] if n.startswith("Gamma_")]) == M
    for name, v in outs[1].items():
        assert np.array_equal(v, outs[2][name]), name


def test_site_range_build_equals_whole_build(cuda):
    """bsg_build_sites (the drop-in MPS step's single call for a site range,
    here sites 10..29 of the M=50 workload, and the two end sites) fed the
    whole build's own cut data gives the whole build's Gammas and Lambdas
    for that range bit for bit."""
    import torch
    from bosonsupremacy_gb300 import _lib, ops, synthetic
    from bosonsupremacy_gb300.pipeline import build_mps
    import ctypes
    cfg = synthetic.MEDIUM
    M, d, chi = cfg.M, cfg.d, cfg.chi
    _, sq = synthetic.lossy_covariances(cfg)
    whole = build_mps(sq, d, chi, precision="split")
    sqd = torch.as_tensor(sq).cuda()
    for s0, s1 in [(10, 30), (0, 1), (M - 1, M)]:
        gam = [torch.empty(chi, chi, d, dtype=torch.complex64, device="cuda") for _ in range(s0, s1)]
        lam = torch.zeros(M - 1, chi, dtype=torch.float64, device="cuda")
        ptrs = (ctypes.c_void_p * len(gam))(*[g.data_ptr() for g in gam])
        h = _lib.Handle.get(0)
        kept = torch.as_tensor(whole.kept).to(torch.int32).cuda()
        _lib.check(_lib.load().bsg_build_sites(h.h, sqd.data_ptr(), M, d, chi, 1e-10, _lib.PREC_SPLIT, _lib.OUT_C64,
                                               s0, s1, whole.res.data_ptr(), whole.num.data_ptr(), whole.S.data_ptr(),
                                               kept.data_ptr(), ptrs, lam.data_ptr(), _lib.stream_ptr()),
                   "bsg_build_sites")
        torch.cuda.synchronize()
        for i in range(s0, s1):
            assert torch.equal(gam[i - s0], whole.Gammas[i]), (s0, s1, i)
            if i < M - 1:
                assert torch.equal(lam[i], whole.Lambdas[i]), (s0, s1, i)
