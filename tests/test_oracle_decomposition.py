"""The covariance-decomposition oracle (oracle/decomposition.py), a CPU
interior-point restatement of get_decomposition.py:16-29's SDP, pinned by
the SDP's closed-form optimum for uniform loss and by its optimality
conditions for mode-dependent loss (no reference output exists: cvxpy and
CVXOPT, which the reference calls, are not installed)."""
import numpy as np
import pytest

from bosonsupremacy_gb300 import synthetic
from oracle import decomposition as D


def symplectic_eigenvalues(X):
    M = X.shape[0] // 2
    ev = np.linalg.eigvals(1j * D.omega(M) @ X)
    return np.sort(np.abs(ev.real))[::2]


@pytest.mark.parametrize("M", [1, 3, 8])
def test_uniform_loss_gives_the_closed_form_pure_part(M):
    cfg = synthetic.GBSConfig("t", M, 4, 16, 0.5, 1.2, 0.35, seed=10 + M)
    cov, sq = synthetic.lossy_covariances(cfg)
    r = D.decompose(cov)
    assert r.rel_gap < 1e-10
    assert np.abs(r.X - sq).max() <= 1e-9 * np.abs(sq).max()


@pytest.mark.parametrize("M", [2, 6])
def test_mode_dependent_loss_optimum_is_pure_feasible_and_certified(M):
    cov = synthetic.nonuniform_lossy_covariance(M, seed=M)
    r = D.decompose(cov)
    X = r.X
    n = 2 * M
    Om = D.omega(M)
    # feasibility of both LMIs (get_decomposition.py:24-25)
    assert np.linalg.eigvalsh(np.block([[X, Om], [-Om, X]]))[0] > -1e-9
    assert np.linalg.eigvalsh(cov - X)[0] > -1e-9
    # a pure state: every symplectic eigenvalue is 1
    assert np.abs(symplectic_eigenvalues(X) - 1.0).max() < 1e-7
    # certificate: dual feasible (Z >= 0, A1*(Z1) - Z2 = I) and zero duality gap
    assert np.linalg.eigvalsh(r.Z1)[0] > -1e-9 and np.linalg.eigvalsh(r.Z2)[0] > -1e-9
    assert np.abs(D.a1_adj(r.Z1) - r.Z2 - np.eye(n)).max() < 1e-9
    assert abs(r.primal_obj - r.dual_obj) <= 1e-9 * (1 + abs(r.primal_obj))


def test_schur_matrix_matches_the_operator_it_represents():
    rng = np.random.default_rng(3)
    n = 6
    def spd(k):
        a = rng.standard_normal((k, k))
        return a @ a.T + k * np.eye(k)
    P1, Z1, P2, Z2 = spd(2 * n), spd(2 * n), spd(n), spd(n)
    idx = D.svec_index(n)
    Msc = D.schur_matrix(P1, Z1, P2, Z2, idx)
    assert np.abs(Msc - Msc.T).max() < 1e-10 * np.abs(Msc).max()
    dX = D.sym(rng.standard_normal((n, n)))
    op = D.a1_adj(D.sym(P1 @ D.a1(dX) @ Z1)) + D.sym(P2 @ dX @ Z2)
    assert np.allclose(D.smat(Msc @ D.svec(dX, idx), n, idx), op, rtol=1e-12, atol=1e-10)
