"""GPU covariance decomposition (bsg_cov_decomposition, the drop-in for
get_decomposition.py:16-29) against the closed-form uniform-loss optimum and
the CPU interior-point oracle, and its blocked Cholesky against numpy."""
import ctypes
import os

import numpy as np
import pytest
import torch

from bosonsupremacy_gb300 import _lib, decomposition, synthetic
from oracle import decomposition as D

pytestmark = pytest.mark.gpu


def potrf(A, cuda):
    t = torch.as_tensor(A).to(cuda).contiguous()
    info = ctypes.c_int(-1)
    _lib.check(_lib.load().bsg_potrf_f64(_lib.Handle.get(0).h, t.data_ptr(), A.shape[0], ctypes.byref(info),
                                         _lib.stream_ptr()), "bsg_potrf_f64")
    return np.tril(t.cpu().numpy()), info.value


@pytest.mark.parametrize("n", [1, 5, 64, 65, 130, 300])
def test_blocked_cholesky_matches_numpy(cuda, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    A = a @ a.T + n * np.eye(n)
    L, info = potrf(A, cuda)
    assert info == 0
    ref = np.linalg.cholesky(A)
    assert np.abs(L - ref).max() <= 1e-12 * np.abs(ref).max()


def test_blocked_cholesky_reports_the_first_bad_pivot(cuda):
    d = np.ones(150)
    d[100] = -1.0
    _, info = potrf(np.diag(d), cuda)
    assert info == 101


@pytest.mark.parametrize("M", [1, 8, 16, 50])
def test_uniform_loss_gives_the_closed_form_pure_part(cuda, M):
    cfg = synthetic.GBSConfig("t", M, 4, 16, 0.6, 1.3, 0.4, seed=20 + M)
    cov, sq = synthetic.lossy_covariances(cfg)
    X, meta = decomposition.decompose(cov)
    assert meta["rel_gap"] < 1e-10 and meta["primal_res"] < 1e-10 and meta["dual_res"] < 1e-10
    assert np.abs(X - sq).max() <= 1e-8 * np.abs(sq).max()


@pytest.mark.parametrize("M", [3, 12])
def test_mode_dependent_loss_matches_the_oracle(cuda, M):
    cov = synthetic.nonuniform_lossy_covariance(M, seed=100 + M)
    X, meta = decomposition.decompose(cov)
    ref = D.decompose(cov)
    assert np.abs(X - ref.X).max() <= 1e-8 * np.abs(ref.X).max()
    assert abs(meta["primal_obj"] - ref.primal_obj) <= 1e-9 * abs(ref.primal_obj)
    Om = D.omega(M)
    assert np.linalg.eigvalsh(np.block([[X, Om], [-Om, X]]))[0] > -1e-9
    assert np.linalg.eigvalsh(cov - X)[0] > -1e-9


def test_cli_writes_and_then_keeps_sq_cov(cuda, tmp_path, capsys):
    cov = synthetic.nonuniform_lossy_covariance(4, seed=7)
    root = str(tmp_path) + "/"
    np.save(root + "cov.npy", cov)
    decomposition.main(["--dir", root])
    sq = np.load(root + "sq_cov.npy")
    assert np.abs(sq - D.decompose(cov).X).max() <= 1e-8 * np.abs(sq).max()
    decomposition.main(["--dir", root])
    assert "already available" in capsys.readouterr().out


def test_bad_shapes_are_rejected(cuda):
    with pytest.raises(ValueError):
        decomposition.decompose(np.eye(5))
