"""Seeded synthetic lossy-GBS covariances (inputs of the MPS construction).

The reference builds ``cov.npy`` from experiment files (make_cov.py:47-135) and
splits it into a pure part ``sq_cov.npy`` plus a thermal/random-displacement
part with a cvxpy SDP (get_decomposition.py:16-29).  Neither the experiment
data nor cvxpy exist here, so inputs are generated:

* a lossless interferometer ``U`` (Haar-random, or a banded brickwork of
  random beam splitters),
* single-mode squeezing ``r_k`` and uniform transmissivity ``eta`` applied as
  pure loss.

Uniform loss commutes with ``U``, so the lossy state is
``O diag(v_x, v_p) O^T`` with ``v_x = eta e^{2r} + 1 - eta`` and
``v_p = eta e^{-2r} + 1 - eta`` (hbar = 2, vacuum = identity), and
``sq_cov = O diag(1/v_p, v_p) O^T`` is an exact pure-state split with
``cov - sq_cov = O diag(v_x - 1/v_p, 0) O^T >= 0``.  ``O`` is the xxpp real
form of ``U``.  Both arrays use the reference's xxpp quadrature order.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Tuple

import numpy as np


@dataclasses.dataclass(frozen=True)
class GBSConfig:
    """One synthetic lossy GBS instance (modes, cutoff, bond dimension)."""

    name: str
    M: int
    d: int
    chi: int
    r_lo: float
    r_hi: float
    eta: float
    banded: bool = False
    band_depth: int = 40
    seed: int = 0

    def label(self) -> str:
        kind = "banded" if self.banded else "haar"
        return f"{self.name}: M={self.M} d={self.d} chi={self.chi} {kind} r~U[{self.r_lo},{self.r_hi}] eta={self.eta}"


# The five workloads (small CPU-runnable case, medium, large single instance,
# 64 uneven instances, largest single-GPU banded case).
SMALL = GBSConfig("M16_d4_chi64", 16, 4, 64, 0.5, 1.0, 0.3)
MEDIUM = GBSConfig("M50_d6_chi256", 50, 6, 256, 0.8, 1.2, 0.4)
LARGE = GBSConfig("M144_d8_chi1024", 144, 8, 1024, 1.2, 1.6, 0.45)
LARGEST = GBSConfig("M216_d10_chi2048_banded", 216, 10, 2048, 1.0, 1.5, 0.33, banded=True)
NAMED = {c.name: c for c in (SMALL, MEDIUM, LARGE, LARGEST)}


def batch_configs(n_instances: int = 64, seed: int = 0) -> List[GBSConfig]:
    """64 independent instances with uneven sizes: M~U{8..48}, d~U{4..8},
    chi in {32,64,128,256}, r~U[0.5,1.4] per instance range, eta~U[0.2,0.6]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_instances):
        M = int(rng.integers(8, 49))
        d = int(rng.integers(4, 9))
        chi = int(rng.choice([32, 64, 128, 256]))
        eta = float(rng.uniform(0.2, 0.6))
        out.append(GBSConfig(f"batch{k}_M{M}_d{d}_chi{chi}", M, d, chi, 0.5, 1.4, eta, seed=seed * 1000 + k + 1))
    return out


def haar_unitary(M: int, rng: np.random.Generator) -> np.ndarray:
    """Haar-random unitary: QR of a complex Ginibre matrix with the phases of
    R's diagonal divided out (Mezzadri's construction)."""
    z = (rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph[None, :]


def banded_unitary(M: int, depth: int, rng: np.random.Generator) -> np.ndarray:
    """Brickwork of ``depth`` layers of random 2x2 beam splitters on neighbouring
    modes; after 40 layers each mode is coupled to the 20 nearest on either side."""
    U = np.eye(M, dtype=np.complex128)
    for layer in range(depth):
        for k in range(layer % 2, M - 1, 2):
            th = rng.uniform(0.0, np.pi / 2)
            ph = rng.uniform(0.0, 2 * np.pi)
            c, s = np.cos(th), np.sin(th)
            bs = np.array([[c, -np.exp(-1j * ph) * s], [np.exp(1j * ph) * s, c]])
            U[[k, k + 1], :] = bs @ U[[k, k + 1], :]
    return U


def passive_symplectic(U: np.ndarray) -> np.ndarray:
    """xxpp real symplectic of the passive map a -> U a (a = (x + i p)/2)."""
    return np.block([[U.real, -U.imag], [U.imag, U.real]])


def lossy_covariances(cfg: GBSConfig, seed: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
    """Return (cov, sq_cov), both 2M x 2M float64 in xxpp order."""
    rng = np.random.default_rng(cfg.seed if seed is None else seed)
    r = rng.uniform(cfg.r_lo, cfg.r_hi, size=cfg.M)
    if cfg.banded:
        U = banded_unitary(cfg.M, cfg.band_depth, rng)
    else:
        U = haar_unitary(cfg.M, rng)
    O = passive_symplectic(U)
    eta = cfg.eta
    vx = eta * np.exp(2 * r) + 1 - eta
    vp = eta * np.exp(-2 * r) + 1 - eta
    cov = O @ np.diag(np.concatenate([vx, vp])) @ O.T
    sq = O @ np.diag(np.concatenate([1.0 / vp, vp])) @ O.T
    cov = 0.5 * (cov + cov.T)
    sq = 0.5 * (sq + sq.T)
    return cov, sq


def nonuniform_lossy_covariance(M: int, seed: int = 0, r_lo: float = 0.5, r_hi: float = 1.2, eta_lo: float = 0.2,
                                eta_hi: float = 0.8) -> np.ndarray:
    """Covariance (2M x 2M, xxpp) with mode-dependent loss between two
    Haar-random interferometers: squeezed vacuum r_k ~ U[r_lo, r_hi] -> U1 ->
    loss eta_k ~ U[eta_lo, eta_hi] on mode k -> U2.  Loss no longer commutes
    with the interferometers, so the pure part has no closed form: this is
    the input the covariance decomposition (an SDP) exists for."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(r_lo, r_hi, size=M)
    O1 = passive_symplectic(haar_unitary(M, rng))
    eta = rng.uniform(eta_lo, eta_hi, size=M)
    O2 = passive_symplectic(haar_unitary(M, rng))
    cov = O1 @ np.diag(np.concatenate([np.exp(2 * r), np.exp(-2 * r)])) @ O1.T
    t = np.sqrt(np.concatenate([eta, eta]))
    cov = t[:, None] * cov * t[None, :] + np.diag(1.0 - t * t)
    cov = O2 @ cov @ O2.T
    return 0.5 * (cov + cov.T)


def write_inputs(cfg: GBSConfig, rootdir: str, seed: Optional[int] = None) -> None:
    """Write ``cov.npy`` and ``sq_cov.npy`` the way make_cov.py:135 and
    get_decomposition.py:30 leave them for kron_cpu.py / MPS_cpu.py."""
    import os

    os.makedirs(rootdir, exist_ok=True)
    cov, sq = lossy_covariances(cfg, seed)
    np.save(os.path.join(rootdir, "cov.npy"), cov)
    np.save(os.path.join(rootdir, "sq_cov.npy"), sq)


def low_photon_patterns(M: int, max_total: int, d: int) -> np.ndarray:
    """All photon patterns [P, M] int32 with at most ``max_total`` photons in
    total and at most d-1 per mode (the pattern sets of the probability and
    correlation checks), ordered by total photon number, then by the sorted
    mode multiset."""
    import itertools

    rows = [np.zeros((1, M), dtype=np.int32)]
    for n in range(1, max_total + 1):
        combos = np.array(list(itertools.combinations_with_replacement(range(M), n)), dtype=np.int64)
        pats = np.zeros((len(combos), M), dtype=np.int32)
        np.add.at(pats, (np.repeat(np.arange(len(combos)), n), combos.ravel()), 1)
        rows.append(pats[(pats <= d - 1).all(axis=1)])
    return np.concatenate(rows)
