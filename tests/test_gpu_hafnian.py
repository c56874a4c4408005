"""GPU parity of the batched hafnian / A_elem seam against the reference's
known answers (tests/golden/hafnian_kat.npz) and the oracle."""
import numpy as np
import pytest

from oracle import reference_mps as R

pytestmark = pytest.mark.gpu

# tolerance per arithmetic: relative to max(|reference|) of the batch
TOL = {"fp64": 1e-12, "split": 1e-10, "fp32": 2e-4}


@pytest.mark.parametrize("prec", ["fp64", "split", "fp32"])
def test_hafnian_matrices_kat(cuda, golden, prec):
    from bosonsupremacy_gb300 import ops
    k = golden("hafnian_kat.npz")
    for n in [0, 1, 2, 3, 4, 5, 6, 8, 10, 12, 14]:
        A = k[f"A_{n}"]
        ref = k[f"haf_{n}"]
        got = ops.hafnian(A, precision=prec).cpu().numpy()
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(got - ref).max() <= TOL[prec] * scale, (n, prec, np.abs(got - ref).max() / scale)


@pytest.mark.parametrize("prec", ["fp64", "split", "fp32"])
def test_a_elem_kat(cuda, golden, prec):
    from bosonsupremacy_gb300 import ops
    k = golden("hafnian_kat.npz")
    Sigma = k["elem_Sigma"]
    for n in [2, 4, 6, 8, 10]:
        tgt, den, ref = k[f"elem_target_{n}"], k[f"elem_den_{n}"], k[f"elem_amp_{n}"]
        got = ops.hafnian_batched(Sigma, tgt, den, precision=prec).cpu().numpy()
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= TOL[prec] * scale, (n, prec)


def test_repeated_targets_vs_oracle(cuda):
    """Heavily repeated indices (the structure of MPS targets) up to n = 20."""
    from bosonsupremacy_gb300 import ops
    rng = np.random.default_rng(5)
    n_len = 12
    X = rng.standard_normal((n_len, n_len)) + 1j * rng.standard_normal((n_len, n_len))
    Sigma = 0.3 * (X + X.T)
    for n in [6, 8, 12, 16, 20]:
        tgt = np.sort(rng.integers(0, 5, size=(16, n)), axis=1).astype(np.int32)
        ref = R.hafnian(R.Sigma_select(Sigma, tgt))
        for prec in ("fp64", "split"):
            got = ops.hafnian_batched(Sigma, tgt, precision=prec).cpu().numpy()
            rel = np.abs(got - ref).max() / np.abs(ref).max()
            assert rel <= (1e-11 if prec == "fp64" else 1e-9), (n, prec, rel)


def test_empty_and_odd(cuda):
    from bosonsupremacy_gb300 import ops
    Sigma = np.eye(4) + 0.5j
    out = ops.hafnian_batched(Sigma, np.zeros((3, 0), np.int32), np.array([1.0, 2.0, 4.0])).cpu().numpy()
    assert np.allclose(out, [1.0, 0.5, 0.25])
    out = ops.hafnian_batched(Sigma, np.zeros((2, 3), np.int32)).cpu().numpy()
    assert np.all(out == 0)


def test_invalid_index_raises(cuda):
    from bosonsupremacy_gb300 import ops
    from bosonsupremacy_gb300._lib import BSGError
    with pytest.raises(BSGError):
        ops.hafnian_batched(np.eye(4), np.array([[0, 9]], np.int32))
