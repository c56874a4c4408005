"""Generate the two large golden fixtures by running the UNMODIFIED reference
scripts (kron_cpu.py, MPS_cpu.py, sampling_cpu.py) from a read-only checkout
of sss441803/BosonSupremacy, with the same mechanical changes as
make_golden.py (np.product shim, FP64 promotion, float16 cast dropped,
sys.argv set, np.random seeded) plus a site filter on MPS_cpu.py's site loop
(MPS_cpu.py:384) for the large workload.

  medium_M50.npz  -- the M=50, d=6, chi=256 workload (Haar, r~U[0.8,1.2],
                     eta=0.4): kron_cpu.py + the whole MPS_cpu.py build,
                     * the Schmidt weights of all 49 cuts,
                     * the probabilities of all 316 251 patterns with <= 4
                       photons, contracted from the reference's Gamma/Lambda
                       (oracle transfer contraction, sampling_cpu.py:75-80
                       with the photon numbers fixed), stored as float32
                       ratios to the largest one (6e-8 relative rounding),
                     * sampling_cpu.py's 10^5 samples (seed 2025, batches of
                       25 000, dd = d + 2): mean, covariance and the first
                       1024 rows, and the sqrtW it drew the displacements with.
                     About 15 minutes on 8 cores (the MPS build is ~8 min).
  large_M144.npz  -- the M=144, d=8, chi=1024 workload (Haar, r~U[1.2,1.6],
                     eta=0.45): kron_cpu.py over all 143 cuts (~7.5 min),
                     * the Schmidt weights of every cut,
                     * the cut files (res, num, S) of cuts 70 and 71,
                     * MPS_cpu.py's site 71 alone (~2.5 min): a stratified
                       sample of its Gamma entries, up to 96 non-zero entries
                       per (j, photon sector) group plus the 64 largest.
  largest_M216.npz -- the M=216, d=10, chi=2048 banded workload (r~U[1.0,1.5],
                     eta=0.33): kron_cpu.py's first 32 cuts (the loop at
                     kron_cpu.py:147 limited to them; ~10 min), their Schmidt
                     weights.

Usage:  python tests/golden/make_golden_large.py REFERENCE_DIR {medium|large|largest|all}
The fixtures are committed next to this script; the GPU machine never needs the
reference itself.
"""
from __future__ import annotations

import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from bosonsupremacy_gb300.synthetic import LARGE, LARGEST, MEDIUM, write_inputs  # noqa: E402
from make_golden import run_ref  # noqa: E402

SAMPLE_SEED = 2025
SAMPLE_N = 100000
SAMPLE_BATCH = 25000
GAMMA_SITE = 71


def _log(msg):
    print(f"[{time.strftime('%H:%M:%S')}] {msg}", flush=True)


def medium(ref: str, out: str) -> None:
    from oracle.reference_mps import enumerate_patterns, pattern_amplitudes  # checker-side helper

    cfg = MEDIUM
    M, d, chi = cfg.M, cfg.d, cfg.chi
    with tempfile.TemporaryDirectory() as tmp:
        root = tmp + "/"
        write_inputs(cfg, root)
        argv = ["--d", str(d), "--chi", str(chi), "--dir", root]
        _log("medium: kron_cpu.py")
        run_ref(ref, "kron_cpu.py", argv, as_main=True)
        _log("medium: MPS_cpu.py (all sites)")
        run_ref(ref, "MPS_cpu.py", argv, as_main=True)
        path = root + f"d_{d}_chi_{chi}/"
        data = {"sq_cov": np.load(root + "sq_cov.npy"), "cov": np.load(root + "cov.npy"),
                "M": M, "d": d, "chi": chi}
        res = np.zeros((M - 1, chi))
        kept = np.zeros(M - 1, np.int32)
        for c in range(M - 1):
            r = np.load(path + f"res_{c}.npy").astype(np.float64)
            res[c, : len(r)] = r
            kept[c] = len(r)
        data["res"] = res
        data["kept"] = kept
        G = [np.load(path + f"Gamma_{i}.npy") for i in range(M)]
        L = [np.load(path + f"Lambda_{i}.npy") for i in range(M - 1)]
        _log("medium: contraction of all <= 4-photon patterns")
        pats = enumerate_patterns(M, 4, d)
        amp = pattern_amplitudes(G, L, pats)
        p = np.abs(amp) ** 2
        pmax = p.max()
        data["pattern_count"] = len(pats)
        data["pattern_prob_max"] = pmax
        data["pattern_prob_rel"] = (p / pmax).astype(np.float32)
        del G, amp
        _log("medium: sampling_cpu.py, 10^5 samples")
        np.random.seed(SAMPLE_SEED)
        sargv = ["--N", str(SAMPLE_N), "--n", str(SAMPLE_BATCH), "--iter", "1", "--d", str(d),
                 "--dd", str(d + 2), "--chi", str(chi), "--dir", root]
        ns = run_ref(ref, "sampling_cpu.py", sargv, as_main=True)
        s = np.load(root + "samples_0.npy")
        data["sqrtW"] = np.asarray(ns["sqrtW"])
        data["sample_seed"] = SAMPLE_SEED
        data["sample_n"] = SAMPLE_N
        data["sample_batch"] = SAMPLE_BATCH
        data["sample_dd"] = d + 2
        data["sample_mean"] = s.astype(np.float64).mean(axis=0)
        data["sample_cov"] = np.cov(s.astype(np.float64).T)
        data["sample_head"] = s[:1024].astype(np.int8)
        np.savez_compressed(out, **data)
        _log(f"medium: wrote {out} ({os.path.getsize(out)} bytes)")


def _gamma_sample(G: np.ndarray, num_r: np.ndarray, num_l: np.ndarray, rng) -> tuple:
    """Up to 96 non-zero entries per (j, |l| + |r|) group and the 64 largest
    entries of a site tensor G[a_{i-1}, a_i, j]."""
    size_r = num_r.reshape(num_r.shape[0], -1).sum(axis=1)
    size_l = num_l.reshape(num_l.shape[0], -1).sum(axis=1)
    picks = []
    for j in range(G.shape[2]):
        nz = np.argwhere(G[:, :, j] != 0)
        if len(nz) == 0:
            continue
        sector = size_r[nz[:, 0]] + size_l[nz[:, 1]]
        for s in np.unique(sector):
            rows = nz[sector == s]
            take = rows[rng.choice(len(rows), size=min(96, len(rows)), replace=False)]
            picks.append(np.column_stack([take, np.full(len(take), j)]))
    flat = np.argsort(np.abs(G).ravel())[-64:]
    picks.append(np.column_stack(np.unravel_index(flat, G.shape)))
    idx = np.unique(np.concatenate(picks).astype(np.int32), axis=0)
    return idx, G[idx[:, 0], idx[:, 1], idx[:, 2]]


def large(ref: str, out: str) -> None:
    cfg = LARGE
    M, d, chi = cfg.M, cfg.d, cfg.chi
    with tempfile.TemporaryDirectory() as tmp:
        root = tmp + "/"
        write_inputs(cfg, root)
        argv = ["--d", str(d), "--chi", str(chi), "--dir", root]
        _log("large: kron_cpu.py (143 cuts)")
        run_ref(ref, "kron_cpu.py", argv, as_main=True)
        path = root + f"d_{d}_chi_{chi}/"
        data = {"sq_cov": np.load(root + "sq_cov.npy"), "M": M, "d": d, "chi": chi}
        res = np.zeros((M - 1, chi))
        kept = np.zeros(M - 1, np.int32)
        for c in range(M - 1):
            r = np.load(path + f"res_{c}.npy").astype(np.float64)
            res[c, : len(r)] = r
            kept[c] = len(r)
        data["res"] = res
        data["kept"] = kept
        for c in (GAMMA_SITE - 1, GAMMA_SITE):
            data[f"num_{c}"] = np.load(path + f"num_{c}.npy")
            data[f"S_{c}"] = np.load(path + f"S_{c}.npy")
        _log(f"large: MPS_cpu.py site {GAMMA_SITE} only")
        site_loop = ("for compute_site in range(M):", f"for compute_site in [{GAMMA_SITE}]:")
        run_ref(ref, "MPS_cpu.py", argv, as_main=True, extra=[site_loop])
        G = np.load(path + f"Gamma_{GAMMA_SITE}.npy")
        idx, val = _gamma_sample(G, data[f"num_{GAMMA_SITE - 1}"], data[f"num_{GAMMA_SITE}"],
                                 np.random.default_rng(71))
        data["gamma_site"] = GAMMA_SITE
        data["gamma_idx"] = idx
        data["gamma_val"] = val
        data["gamma_absmax"] = np.abs(G).max()
        data["gamma_nonzero"] = int(np.count_nonzero(G))
        np.savez_compressed(out, **data)
        _log(f"large: wrote {out} ({os.path.getsize(out)} bytes, {len(idx)} Gamma entries)")


LARGEST_CUTS = 32


def largest(ref: str, out: str) -> None:
    cfg = LARGEST
    M, d, chi = cfg.M, cfg.d, cfg.chi
    with tempfile.TemporaryDirectory() as tmp:
        root = tmp + "/"
        write_inputs(cfg, root)
        argv = ["--d", str(d), "--chi", str(chi), "--dir", root]
        _log(f"largest: kron_cpu.py, cuts 0..{LARGEST_CUTS - 1}")
        cut_loop = ("for compute_site in range(M - 1):", f"for compute_site in range({LARGEST_CUTS}):")
        run_ref(ref, "kron_cpu.py", argv, as_main=True, extra=[cut_loop])
        path = root + f"d_{d}_chi_{chi}/"
        res = np.zeros((LARGEST_CUTS, chi))
        kept = np.zeros(LARGEST_CUTS, np.int32)
        for c in range(LARGEST_CUTS):
            r = np.load(path + f"res_{c}.npy").astype(np.float64)
            res[c, : len(r)] = r
            kept[c] = len(r)
        np.savez_compressed(out, sq_cov=np.load(root + "sq_cov.npy"), M=M, d=d, chi=chi, res=res, kept=kept)
        _log(f"largest: wrote {out} ({os.path.getsize(out)} bytes)")


def main():
    which_all = ("medium", "large", "largest", "all")
    if len(sys.argv) != 3 or sys.argv[2] not in which_all:
        sys.exit("usage: make_golden_large.py REFERENCE_DIR {medium|large|largest|all}")
    ref, which = sys.argv[1], sys.argv[2]
    if which in ("medium", "all"):
        medium(ref, os.path.join(HERE, "medium_M50.npz"))
    if which in ("large", "all"):
        large(ref, os.path.join(HERE, "large_M144.npz"))
    if which in ("largest", "all"):
        largest(ref, os.path.join(HERE, "largest_M216.npz"))


if __name__ == "__main__":
    main()
