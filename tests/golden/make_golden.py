"""Generate the golden fixtures in this folder by running the UNMODIFIED
reference scripts (kron_cpu.py, MPS_cpu.py, sampling_cpu.py) from a
read-only checkout of sss441803/BosonSupremacy.

The reference is executed from its own source text with four mechanical
changes, the same ones the oracle's header names:
  * ``np.product = np.prod`` (removed in numpy 2.x; MPS_cpu.py:413, 437, 468, 479),
  * FP64 promotion: 'complex64' -> 'complex128', 'float32' -> 'float64'
    (MPS_cpu.py:17, 123, 126, 337, 351, 397-398, 488; sampling_cpu.py:55, 77),
  * the float16 cast of the Schmidt weights dropped (kron_cpu.py:127),
  * ``sys.argv`` set before exec (module-level argparse) and np.random seeded
    before the sampler (it is unseeded, sampling_cpu.py:37, 52, 92).

Usage:  python tests/golden/make_golden.py REFERENCE_DIR
The fixtures are small .npz files committed next to this script; the GPU machine
never needs the reference itself.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from bosonsupremacy_gb300.synthetic import GBSConfig, SMALL, lossy_covariances, write_inputs  # noqa: E402

FP64 = [("'complex64'", "'complex128'"), ("'float32'", "'float64'"),
        ("res.astype('float16')", "res")]

# Tiny instance whose full kron + MPS output fits a fixture.
TINY = GBSConfig("M8_d4_chi24", 8, 4, 24, 0.5, 1.0, 0.3, seed=7)


def _source(ref: str, name: str, extra=()) -> str:
    with open(os.path.join(ref, name)) as f:
        src = f.read()
    for a, b in list(FP64) + list(extra):
        if a not in src and (a, b) in extra:
            raise ValueError(f"{name}: substitution target not found: {a!r}")
        src = src.replace(a, b)
    return src


def run_ref(ref: str, name: str, argv, as_main: bool, extra=()):
    """exec one reference script; returns its namespace.  ``extra`` holds
    further (old, new) source substitutions (e.g. a site filter)."""
    np.product = np.prod  # numpy 2.x shim
    ns = {"__name__": "__main__" if as_main else "ref_" + name[:-3]}
    old = sys.argv
    sys.argv = [name] + list(argv)
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            exec(compile(_source(ref, name, extra), os.path.join(ref, name), "exec"), ns)
    finally:
        sys.argv = old
    return ns


def hafnian_kat(ref: str, out: str) -> None:
    """Known-answer vectors for the batched hafnian and A_elem (MPS_cpu.py:117-187, 334-355)."""
    ns = run_ref(ref, "MPS_cpu.py", ["--d", "4", "--chi", "8", "--dir", "/nonexistent/"], as_main=False)
    rng = np.random.default_rng(123)
    data = {}
    for n in [0, 1, 2, 3, 4, 5, 6, 8, 10, 12, 14]:
        B = 6
        X = rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))
        A = 0.5 * (X + np.transpose(X, (0, 2, 1)))
        data[f"A_{n}"] = A
        data[f"haf_{n}"] = np.asarray(ns["hafnian"](A.astype(np.complex128)))
    # A_elem with a repeated-index gather from one symmetric Sigma
    n_len = 20
    X = rng.standard_normal((n_len, n_len)) + 1j * rng.standard_normal((n_len, n_len))
    Sigma = 0.25 * (X + X.T)
    for n in [2, 4, 6, 8, 10]:
        tgt = np.sort(rng.integers(0, n_len, size=(40, n)), axis=1).astype(np.int32)
        den = rng.uniform(0.5, 2.0, size=40)
        amp, _, _ = ns["A_elem"](Sigma, tgt, den, 0.5)
        data[f"elem_target_{n}"] = tgt
        data[f"elem_den_{n}"] = den
        data[f"elem_amp_{n}"] = np.asarray(amp)
    data["elem_Sigma"] = Sigma
    np.savez_compressed(out, **data)


def pipeline(ref: str, cfg: GBSConfig, full_gamma: bool, n_samples: int, out: str, n_big: int = 0,
             big_batch: int = 25000) -> None:
    """kron_cpu.py + MPS_cpu.py on one synthetic instance; optionally the
    sampler (n_samples in one batch, seed 2024; and n_big in batches of
    big_batch, seed 2025, for the one- and two-point correlations)."""
    from oracle.reference_mps import enumerate_patterns, pattern_amplitudes  # checker-side helper

    with tempfile.TemporaryDirectory() as tmp:
        root = tmp + "/"
        write_inputs(cfg, root)
        argv = ["--d", str(cfg.d), "--chi", str(cfg.chi), "--dir", root]
        run_ref(ref, "kron_cpu.py", argv, as_main=True)
        run_ref(ref, "MPS_cpu.py", argv, as_main=True)
        path = root + f"d_{cfg.d}_chi_{cfg.chi}/"
        M = cfg.M
        data = {"sq_cov": np.load(root + "sq_cov.npy"), "cov": np.load(root + "cov.npy"),
                "M": M, "d": cfg.d, "chi": cfg.chi}
        G = [np.load(path + f"Gamma_{i}.npy") for i in range(M)]
        L = [np.load(path + f"Lambda_{i}.npy") for i in range(M - 1)]
        for c in range(M - 1):
            data[f"res_{c}"] = np.load(path + f"res_{c}.npy")
            data[f"num_{c}"] = np.load(path + f"num_{c}.npy")
            data[f"S_{c}"] = np.load(path + f"S_{c}.npy")
            data[f"Lambda_{c}"] = L[c]
        if full_gamma:
            for i in range(M):
                data[f"Gamma_{i}"] = G[i]
            # Sigma and Z of every site from the reference's own functions
            ns = run_ref(ref, "MPS_cpu.py", argv, as_main=False)
            sq_cov = data["sq_cov"]
            S_full = ns["williamson"](sq_cov)[1]
            for i in range(M):
                if i == 0:
                    S_l, S_r = data["S_0"], S_full
                elif i == M - 1:
                    S_l, S_r = np.zeros((0, 0)), data[f"S_{M - 2}"]
                else:
                    S_l, S_r = data[f"S_{i}"], data[f"S_{i - 1}"]
                U2, sq, U1 = ns["get_U2_sq_U1"](S_l, S_r)
                data[f"Sigma_{i}"] = ns["get_Sigma"](U2, sq, U1)
                data[f"Z_{i}"] = np.sqrt(np.prod(np.cosh(sq)))
        pats = enumerate_patterns(M, 4 if M <= 16 else 3, cfg.d)
        amp = pattern_amplitudes(G, L, pats)
        data["patterns"] = pats
        data["pattern_probs"] = np.abs(amp) ** 2
        if n_samples:
            np.random.seed(2024)
            sargv = ["--N", str(n_samples), "--n", str(n_samples), "--iter", "1", "--d", str(cfg.d),
                     "--dd", str(cfg.d + 2), "--chi", str(cfg.chi), "--dir", root]
            run_ref(ref, "sampling_cpu.py", sargv, as_main=True)
            s = np.load(root + "samples_0.npy").astype(np.float64)
            data["sample_seed"] = 2024
            data["sample_dd"] = cfg.d + 2
            data["sample_n"] = n_samples
            data["sample_mean"] = s.mean(axis=0)
            data["sample_cov"] = np.cov(s.T)
            data["sample_head"] = s[:64].astype(np.int8)
        if n_big:
            np.random.seed(2025)
            sargv = ["--N", str(n_big), "--n", str(big_batch), "--iter", "1", "--d", str(cfg.d),
                     "--dd", str(cfg.d + 2), "--chi", str(cfg.chi), "--dir", root]
            run_ref(ref, "sampling_cpu.py", sargv, as_main=True)
            s = np.load(root + "samples_0.npy").astype(np.float64)
            data["big_sample_seed"] = 2025
            data["big_sample_n"] = n_big
            data["big_sample_batch"] = big_batch
            data["big_sample_mean"] = s.mean(axis=0)
            data["big_sample_cov"] = np.cov(s.T)
            data["big_sample_head"] = s[:256].astype(np.int8)
        np.savez_compressed(out, **data)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_DIR")
    ref = sys.argv[1]
    hafnian_kat(ref, os.path.join(HERE, "hafnian_kat.npz"))
    pipeline(ref, TINY, full_gamma=True, n_samples=2000, out=os.path.join(HERE, "tiny_M8.npz"))
    pipeline(ref, SMALL, full_gamma=False, n_samples=10000, out=os.path.join(HERE, "small_M16.npz"), n_big=100000)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
