"""Mathematical facts the GPU design relies on, checked on the CPU against
the oracle: the repetition-aware hafnian recurrence, the closed-form Sigma,
pruning to chi per step, and the brute-force hafnian."""
import functools
from math import factorial

import numpy as np

from oracle import reference_mps as R


def multiset_hafnian(Sigma, target):
    """F_m = (1/m_a) sum_b A_ab F_{m-e_a-e_b}; haf = prod m! F_m (classes in
    ascending multiplicity, a = first non-empty class) -- the recurrence the
    partition programs of bsg_programs.cpp encode."""
    vals, counts = np.unique(target, return_counts=True)
    order = np.argsort(counts, kind="stable")
    cls, m = vals[order], counts[order]
    A = Sigma[np.ix_(cls, cls)]
    k = len(cls)

    @functools.lru_cache(None)
    def F(r):
        if sum(r) == 0:
            return 1.0 + 0j
        a = next(i for i, x in enumerate(r) if x > 0)
        acc = 0j
        for b in range(a, k):
            if r[b] == 0 or (b == a and r[a] < 2):
                continue
            s = list(r)
            s[a] -= 1
            s[b] -= 1
            acc += A[a, b] * F(tuple(s))
        return acc / r[a]

    return F(tuple(int(x) for x in m)) * np.prod([factorial(int(x)) for x in m])


def test_multiset_recurrence_equals_reference_hafnian():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((10, 10)) + 1j * rng.standard_normal((10, 10))
    S = 0.4 * (X + X.T)
    for n in [2, 4, 6, 8, 10, 12]:
        for _ in range(10):
            t = rng.integers(0, 6, size=n)
            ref = R.hafnian(R.Sigma_select(S, t[None].astype(np.int32)))[0]
            assert abs(multiset_hafnian(S, t) - ref) <= 1e-12 * max(1.0, abs(ref))


def test_bruteforce_hafnian():
    rng = np.random.default_rng(2)
    for n in [2, 4, 6, 8]:
        X = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        A = X + X.T
        assert abs(R.hafnian(A[None])[0] - R.hafnian_bruteforce(A)) < 1e-10 * abs(R.hafnian_bruteforce(A))


def test_closed_form_sigma(golden):
    """Sigma = [[B X, X^T], [X, -X conj B]], X = conj(A)^-1, Z = sqrt|det A|
    for S = (1 (+) S_l)^-1 S_r equals the reference's Bloch-Messiah route."""
    t = golden("tiny_M8.npz")
    M = int(t["M"])
    for i in range(1, M):
        S_l = t[f"S_{i}"] if i < M - 1 else np.zeros((0, 0))
        S_r = t[f"S_{i - 1}"]
        Mr = S_r.shape[0] // 2
        inner = np.concatenate([np.arange(1, Mr), np.arange(1, Mr) + Mr])
        Li = np.eye(2 * Mr)
        if S_l.size:
            n = S_l.shape[0] // 2
            a, b, c, e = S_l[:n, :n], S_l[:n, n:], S_l[n:, :n], S_l[n:, n:]
            Li[np.ix_(inner, inner)] = np.block([[e.T, -b.T], [-c.T, a.T]])
        S = Li @ S_r
        xx, xp, px, pp = S[:Mr, :Mr], S[:Mr, Mr:], S[Mr:, :Mr], S[Mr:, Mr:]
        A = 0.5 * (xx + pp + 1j * (px - xp))
        B = 0.5 * (xx - pp + 1j * (px + xp))
        X = np.linalg.inv(A.conj())
        Sig = np.block([[B @ X, X.T], [X, -X @ B.conj()]])
        assert np.abs(Sig - t[f"Sigma_{i}"]).max() < 1e-12, i
        assert abs(np.sqrt(abs(np.linalg.det(A))) - float(t[f"Z_{i}"])) < 1e-12 * float(t[f"Z_{i}"]), i


def test_pruning_to_chi_selects_the_same_cut(golden):
    t = golden("small_M16.npz")
    sq, d, chi = t["sq_cov"], int(t["d"]), int(t["chi"])
    for L in (1, 4, 9):
        a = R.get_cumsum_kron(sq, L, chi=chi, max_dim=10 ** 5, cutoff=d)
        b = R.get_cumsum_kron(sq, L, chi=chi, max_dim=chi, cutoff=d)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_williamson_rejects_invalid_input():
    import pytest
    with pytest.raises(ValueError, match="not symmetric"):
        R.williamson(np.array([[2.0, 1.0], [0.0, 2.0]]))
    with pytest.raises(ValueError, match="positive definite"):
        R.williamson(-np.eye(2))
