"""CPU oracle for the covariance decomposition (test infrastructure only).

get_decomposition.py:16-29 splits the experiment covariance ``cov`` (2M x 2M,
xxpp) into a pure quantum part and classical noise with the semidefinite
program

    minimise tr X  subject to  [[X, Omega], [-Omega, X]] >= 0,  cov - X >= 0,

Omega = kron([[0, 1], [-1, 0]], I_M) (get_decomposition.py:18-26), solved by
cvxpy with the CVXOPT interior-point solver (:27) and saved as sq_cov.npy (:30).
cvxpy and CVXOPT are not installed here, so this module restates the
problem's solution method from the published algorithm instead: a primal-dual
interior-point method with the HKM search direction (Helmberg, Rendl,
Vanderbei and Wolkowicz 1996; Kojima, Shindoh and Hara 1997; Monteiro 1997)
and Mehrotra's predictor-corrector step (Mehrotra 1992; centring kept >= 0.1),
on the same real formulation -- two LMI blocks, S1 = [[X, Omega], [-Omega, X]]
(2n x 2n, n = 2M) and S2 = cov - X (n x n).

The optimum is unique (a pure state); the iterates stay near the central path
and reach it to about the duality gap.  For uniform loss it is known in
closed form (the pure part O diag(1/v_p, v_p) O^T of a passive O applied to
lossy squeezed modes), which pins this solver; for mode-dependent loss its
primal-dual pair certifies itself (feasibility, zero gap).  Nothing in the
package imports this file.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.linalg as sla


def omega(M: int) -> np.ndarray:
    """Omega = kron([[0, 1], [-1, 0]], I_M) (get_decomposition.py:18-20)."""
    return np.kron(np.array([[0.0, 1.0], [-1.0, 0.0]]), np.eye(M))


def svec_index(n: int):
    """Upper-triangle index pairs (i <= j) of the symmetric basis and the
    basis scales alpha (1/sqrt(2) off the diagonal, 1/2 on it), so that
    E_a = alpha_a (e_i e_j^T + e_j e_i^T) is orthonormal."""
    i, j = np.triu_indices(n)
    alpha = np.where(i == j, 0.5, 1.0 / np.sqrt(2.0))
    return i, j, alpha


def svec(A: np.ndarray, idx) -> np.ndarray:
    i, j, alpha = idx
    return 2.0 * alpha * A[i, j]


def smat(v: np.ndarray, n: int, idx) -> np.ndarray:
    """sum_a v_a E_a (inverse of svec)."""
    i, j, alpha = idx
    w = np.where(i == j, 1.0, alpha) * v
    A = np.zeros((n, n))
    A[i, j] = w
    A[j, i] = w
    return A


def sym(A: np.ndarray) -> np.ndarray:
    return 0.5 * (A + A.T)


def a1(X: np.ndarray) -> np.ndarray:
    """A1(X) = [[X, 0], [0, X]]."""
    n = X.shape[0]
    out = np.zeros((2 * n, 2 * n))
    out[:n, :n] = X
    out[n:, n:] = X
    return out


def a1_adj(Z: np.ndarray) -> np.ndarray:
    """Adjoint of A1: the sum of the two diagonal blocks."""
    n = Z.shape[0] // 2
    return Z[:n, :n] + Z[n:, n:]


def schur_matrix(P1, Z1, P2, Z2, idx) -> np.ndarray:
    """HKM Schur complement in the svec basis:
    M_ab = tr(A1(E_a) P1 A1(E_b) Z1) + tr(E_a P2 E_b Z2), with
    tr(E_a P E_b Z) = alpha_a alpha_b (P_jk Z_li + P_jl Z_ki + P_ik Z_lj + P_il Z_kj)
    for a = (i, j), b = (k, l)."""
    i, j, alpha = idx
    n = P2.shape[0]
    pairs = [(P1[p * n:(p + 1) * n, q * n:(q + 1) * n], Z1[q * n:(q + 1) * n, p * n:(p + 1) * n])
             for p in range(2) for q in range(2)] + [(P2, Z2)]
    I, J, K, L = i[:, None], j[:, None], i[None, :], j[None, :]
    out = np.zeros((len(i), len(i)))
    for P, Z in pairs:
        out += P[J, K] * Z[L, I] + P[J, L] * Z[K, I] + P[I, K] * Z[L, J] + P[I, L] * Z[K, J]
    return out * (alpha[:, None] * alpha[None, :])


def max_step(S: np.ndarray, dS: np.ndarray, tau: float) -> float:
    """Largest step in [0, 1] keeping S + a dS positive definite (a fraction
    tau of the way to the boundary)."""
    L = np.linalg.cholesky(S)
    B = sla.solve_triangular(L, sla.solve_triangular(L, dS, lower=True).T, lower=True)
    lam = np.linalg.eigvalsh(sym(B))[0]
    return 1.0 if lam >= 0 else min(1.0, tau / -lam)


@dataclasses.dataclass
class Result:
    X: np.ndarray
    iterations: int
    primal_obj: float
    dual_obj: float
    rel_gap: float
    primal_res: float
    dual_res: float
    Z1: np.ndarray
    Z2: np.ndarray


def decompose(cov: np.ndarray, tol: float = 1e-10, max_iter: int = 100) -> Result:
    """min tr X s.t. [[X, Omega], [-Omega, X]] >= 0, cov - X >= 0
    (get_decomposition.py:22-27) by an infeasible-start HKM primal-dual
    interior-point method with Mehrotra's predictor-corrector."""
    V = 0.5 * (np.asarray(cov, dtype=np.float64) + np.asarray(cov, dtype=np.float64).T)
    n = V.shape[0]
    M = n // 2
    C1 = np.zeros((2 * n, 2 * n))
    Om = omega(M)
    C1[:n, n:] = Om
    C1[n:, :n] = -Om
    idx = svec_index(n)
    nu = 3 * n  # barrier dimension: blocks of order 2n and n
    xi = max(10.0, np.sqrt(n), np.abs(V).max() * np.sqrt(n))
    X = np.zeros((n, n))
    S1, S2 = xi * np.eye(2 * n), xi * np.eye(n)
    Z1, Z2 = xi * np.eye(2 * n), xi * np.eye(n)
    tau = 0.98
    it = 0
    for it in range(1, max_iter + 1):
        Rp1 = S1 - a1(X) - C1
        Rp2 = S2 - V + X
        Rd = a1_adj(Z1) - Z2 - np.eye(n)
        pobj = np.trace(X)
        dobj = -np.sum(Z1 * C1) - np.sum(Z2 * V)
        gap = np.sum(S1 * Z1) + np.sum(S2 * Z2)
        mu = gap / nu
        rel_gap = gap / (1.0 + abs(pobj) + abs(dobj))
        pres = max(np.linalg.norm(Rp1), np.linalg.norm(Rp2)) / (1.0 + np.linalg.norm(V))
        dres = np.linalg.norm(Rd) / (1.0 + np.sqrt(n))
        if rel_gap < tol and pres < tol and dres < tol:
            break
        P1, P2 = np.linalg.inv(S1), np.linalg.inv(S2)
        P1, P2 = sym(P1), sym(P2)
        Msc = schur_matrix(P1, Z1, P2, Z2, idx)
        cf = sla.cho_factor(Msc)

        def direction(G1, G2):
            rhs = Rd + a1_adj(G1) + a1_adj(sym(P1 @ Rp1 @ Z1)) - G2 - sym(P2 @ Rp2 @ Z2)
            dX = smat(sla.cho_solve(cf, svec(sym(rhs), idx)), n, idx)
            dS1 = a1(dX) - Rp1
            dS2 = -dX - Rp2
            dZ1 = G1 - sym(P1 @ dS1 @ Z1)
            dZ2 = G2 - sym(P2 @ dS2 @ Z2)
            return dX, dS1, dS2, dZ1, dZ2

        # predictor (sigma = 0)
        dX, dS1, dS2, dZ1, dZ2 = direction(-Z1, -Z2)
        ap = min(max_step(S1, dS1, 1.0), max_step(S2, dS2, 1.0))
        ad = min(max_step(Z1, dZ1, 1.0), max_step(Z2, dZ2, 1.0))
        mu_aff = (np.sum((S1 + ap * dS1) * (Z1 + ad * dZ1)) + np.sum((S2 + ap * dS2) * (Z2 + ad * dZ2))) / nu
        # Mehrotra's sigma, kept >= 0.1 so the iterates stay near the central
        # path: X then converges linearly in the gap (pure Mehrotra steps
        # leave X about sqrt(gap) from the optimum for mode-dependent loss)
        sigma = max(0.1, min(1.0, (mu_aff / mu) ** 3))
        # corrector
        G1 = sigma * mu * P1 - Z1 - sym(P1 @ dS1 @ dZ1)
        G2 = sigma * mu * P2 - Z2 - sym(P2 @ dS2 @ dZ2)
        dX, dS1, dS2, dZ1, dZ2 = direction(G1, G2)
        ap = min(max_step(S1, dS1, tau), max_step(S2, dS2, tau))
        ad = min(max_step(Z1, dZ1, tau), max_step(Z2, dZ2, tau))
        X = X + ap * dX
        S1 = sym(S1 + ap * dS1)
        S2 = sym(S2 + ap * dS2)
        Z1 = sym(Z1 + ad * dZ1)
        Z2 = sym(Z2 + ad * dZ2)
    return Result(sym(X), it, pobj, dobj, rel_gap, pres, dres, Z1, Z2)
