"""Drop-in for sampling_cpu.py: photon-number samples of the MPS on the GPU.

    python -m bosonsupremacy_gb300.sampling --N N --n n --iter I --d D --dd DD --chi CHI --dir ROOT/
        [--precision split|fp64|fp32]

Same flags (sampling_cpu.py:7-15), inputs (ROOT/sq_cov.npy, ROOT/cov.npy,
ROOT/d_{D}_chi_{CHI}/Gamma_i.npy and Lambda_i.npy) and outputs
(ROOT/samples_{iter}.npy, int64 [N, M]; sampling_cpu.py:176-183).  The random
numbers come from numpy's global generator in the reference's order -- one
normal(size=(2M, n)) per batch, then one rand(n, 1) per site -- so with the
same np.random.seed the samples are the reference's, draw for draw (up to
thresholds that fall within rounding of a cumulative probability).

Function-level mirror: ``sampling(path, dd, Lambda, sqrtW, samples_in_parallel)``
(sampling_cpu.py:30-117), ``batch_displaces(N, alphas)`` (:133-148),
``displace``/``displaces`` (:124-131), ``mu_to_alpha``/``batch_mu_to_alpha``
(:150-159) and ``thermal_sqrtW(cov, sq_cov)`` (:166-170).  The chain
contraction, displacements, probabilities and draws all run in libbsg.
"""
from __future__ import annotations

import argparse
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import ops


def mu_to_alpha(mu, hbar=2):
    """Mean displacement of each mode (sampling_cpu.py:150-154)."""
    M = len(mu) // 2
    return (mu[:M] + 1j * mu[M:]) / np.sqrt(2 * hbar)


def batch_mu_to_alpha(mu, hbar=2):
    """Per-sample mean displacements [n, M] (sampling_cpu.py:156-159)."""
    M = mu.shape[1] // 2
    return (mu[:, :M] + 1j * mu[:, M:]) / np.sqrt(2 * hbar)


def batch_displaces(N, alphas, device: int = 0) -> np.ndarray:
    """D(alpha) for alphas [n, M]: complex128 [n, M, N, N] (sampling_cpu.py:133-148)."""
    return ops.displacements(np.asarray(alphas, dtype=np.complex128), N, device=device).cpu().numpy()


def displaces(N, alphas, device: int = 0) -> np.ndarray:
    """D(alpha) for a 1-d batch of alphas (sampling_cpu.py:128-131)."""
    return batch_displaces(N, np.asarray(alphas).reshape(-1), device=device)


def displace(N, alpha, device: int = 0) -> np.ndarray:
    """D(alpha) in N dimensions (sampling_cpu.py:124-126)."""
    return batch_displaces(N, np.asarray([alpha]), device=device)[0]


def thermal_sqrtW(cov, sq_cov) -> np.ndarray:
    """Cholesky factor of the thermal part cov - sq_cov, shifted to be
    positive definite as the reference does (sampling_cpu.py:168-170;
    host-side setup of a 2M x 2M matrix).

    The thermal part of a uniform-loss state has rank M, so the reference's
    shift 1.000001 |lambda_min| only works where LAPACK returns a negative
    lambda_min; where it returns zero or a positive rounding value the shift
    is doubled from 1e-15 |T| until the factorisation succeeds.  The
    difference reaches the samples through sqrt(shift) ~ 1e-8 relative
    changes of the displacements."""
    thermal = np.asarray(cov) - np.asarray(sq_cov)
    eye = np.eye(len(thermal))
    shift = 1.000001 * np.abs(np.min(np.linalg.eigvalsh(thermal)))
    try:
        return np.linalg.cholesky(thermal + shift * eye)
    except np.linalg.LinAlgError:
        pass
    shift = max(shift, 1e-15 * max(1.0, float(np.abs(thermal).max())))
    for _ in range(64):
        try:
            return np.linalg.cholesky(thermal + shift * eye)
        except np.linalg.LinAlgError:
            shift *= 2.0
    raise np.linalg.LinAlgError("thermal covariance is not positive semi-definite")


def draw_random(M: int, n: int, rng=np.random):
    """The random numbers of one batch in the reference's draw order:
    normals [2M, n] (sampling_cpu.py:37), then thresholds [M, n], one
    rand(n, 1) per site (:52, :92)."""
    z = rng.normal(size=(2 * M, n))
    u = np.stack([rng.rand(n, 1)[:, 0] for _ in range(M)])
    return z, u


def sample_mps(Gammas: Sequence[torch.Tensor], Lambdas, sqrtW, dd: int, n: int, rng=np.random, precision="split",
               device: int = 0) -> np.ndarray:
    """n samples [n, M] int64 of the MPS (Gammas [chi, chi, d] per site,
    Lambdas [M-1, chi]) with random numbers drawn from `rng`."""
    M = len(Gammas)
    z, u = draw_random(M, n, rng)
    return ops.sample(Gammas, Lambdas, sqrtW, z, u, dd, precision=precision, device=device).cpu().numpy()


def sampling(path, dd, Lambda, sqrtW, samples_in_parallel, compare=False, precision="split",
             gammas: Optional[List[torch.Tensor]] = None, device: int = 0) -> np.ndarray:
    """sampling_cpu.py:30-117 with the same arguments: Gamma_i.npy read from
    `path`, Lambda [chi, M-1], sqrtW [2M, 2M]; returns [n, M] int64.
    `gammas` may carry the device tensors across batches."""
    M = len(sqrtW) // 2
    dev = torch.device("cuda", device)
    if gammas is None:
        want = torch.complex128 if precision == "fp64" else torch.complex64
        gammas = [torch.as_tensor(np.load(path + f"Gamma_{i}.npy")).to(dev, want) for i in range(M)]
    lam = np.ascontiguousarray(np.asarray(Lambda, dtype=np.float64).T)
    return sample_mps(gammas, lam, sqrtW, dd, samples_in_parallel, np.random, precision, device)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--N", type=int, help="Total number of samples.")
    p.add_argument("--n", type=int, help="Number of samples per batch.")
    p.add_argument("--iter", type=int, help="Number of iterations of sampling.")
    p.add_argument("--d", type=int, help="d of the MPS (photons per mode before displacement - 1).")
    p.add_argument("--dd", type=int, help="d after random displacement (photons that can be sampled - 1).")
    p.add_argument("--chi", type=int, help="Bond dimension.")
    p.add_argument("--dir", type=str, help="Root directory.", default="0")
    p.add_argument("--precision", default="split", choices=["split", "fp64", "fp32"])
    args = p.parse_args(argv)
    rootdir = args.dir
    path = rootdir + f"d_{args.d}_chi_{args.chi}/"
    sq_cov = np.load(rootdir + "sq_cov.npy")
    cov = np.load(rootdir + "cov.npy")
    sqrtW = thermal_sqrtW(cov, sq_cov)
    M = sqrtW.shape[0] // 2
    Lambda = np.zeros([args.chi, M - 1], dtype="float32")
    for i in range(M - 1):
        Lambda[:, i] = np.load(path + f"Lambda_{i}.npy")
    want = torch.complex128 if args.precision == "fp64" else torch.complex64
    gammas = [torch.as_tensor(np.load(path + f"Gamma_{i}.npy")).to("cuda", want) for i in range(M)]
    for it in range(args.iter):
        samples = np.zeros([0, M], dtype="int8")
        for begin in range(0, args.N, args.n):
            end = min(args.N, begin + args.n)
            sub = sampling(path, args.dd, Lambda, sqrtW, end - begin, precision=args.precision, gammas=gammas)
            samples = np.concatenate([samples, sub], axis=0)
            np.save(rootdir + f"samples_{it}.npy", samples)


if __name__ == "__main__":
    main()
