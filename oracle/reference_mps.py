"""ORACLE -- test infrastructure only, never the product.

CPU restatement (numpy/scipy, FP64 throughout) of the reference's MPS
construction for lossy Gaussian boson sampling (sss441803/BosonSupremacy):

* per-cut truncation to bond dimension chi      kron_cpu.py:46-127
* per-site Gamma/Lambda build (batched hafnians) MPS_cpu.py:19-525
* the sampler that consumes Gamma/Lambda          sampling_cpu.py:30-159

The reference runs in complex64/float32 and saves Schmidt weights as float16
(MPS_cpu.py:17, 397-398; kron_cpu.py:127).  This restatement is the
FP64-promoted form of the same algorithm: every array is complex128/float64
and the float16 cast is dropped.  It is pinned against outputs of the
unmodified reference (with exactly those dtype promotions) by the fixtures
in ``tests/golden``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module, and only as the checker.
"""
from __future__ import annotations

import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
from scipy.linalg import block_diag, schur, sqrtm, svd, expm
from scipy.special import factorial

CDT = np.complex128


# ----------------------------------------------------------------------------
# Williamson decomposition  (MPS_cpu.py:49-115 == kron_cpu.py:23-89)
# ----------------------------------------------------------------------------
def _omega(n: int) -> np.ndarray:
    """xxpp symplectic form [[0, I], [-I, 0]] (MPS_cpu.py:49-53)."""
    z = np.zeros((n, n))
    e = np.eye(n)
    return np.block([[z, e], [-e, z]])


def _xpxp_order(two_n: int) -> np.ndarray:
    """Index list that reorders xpxp -> xxpp (MPS_cpu.py:55-70)."""
    return np.arange(two_n).reshape(-1, 2).T.reshape(-1)


def williamson(V: np.ndarray, tol: float = 1e-11) -> Tuple[np.ndarray, np.ndarray]:
    """Return (Db, S) with V = S Db S^T, Db = diag(nu, nu) (MPS_cpu.py:72-115).

    Same steps as the reference: V^{-1/2} by sqrtm(inv V), real Schur form of
    the antisymmetric V^{-1/2} Omega V^{-1/2}, 2x2 blocks oriented so that the
    upper entry is positive, xpxp -> xxpp reordering, S = inv(V^{-1/2} K Db^{1/2})^T.
    Raises ValueError with the reference's messages on invalid input.
    """
    n2, m2 = V.shape
    if n2 != m2:
        raise ValueError("The input matrix is not square")
    if np.linalg.norm(V - V.T) >= tol:
        raise ValueError("The input matrix is not symmetric")
    if n2 % 2:
        raise ValueError("The input matrix must have an even number of rows/columns")
    n = n2 // 2
    if np.any(np.linalg.eigvalsh(V) <= 0):
        raise ValueError("Input matrix is not positive definite")
    w = sqrtm(np.linalg.inv(V)).real
    t, K = schur(w @ _omega(n) @ w)
    flip = np.array([[0.0, 1.0], [1.0, 0.0]])
    p = block_diag(*[np.eye(2) if t[2 * i, 2 * i + 1] > 0 else flip for i in range(n)])
    Kp = K @ p
    tp = p @ t @ p
    order = _xpxp_order(n2)
    t_xxpp = tp[:, order][order]
    K_xxpp = Kp[:, order]
    inv_nu = np.array([1.0 / t_xxpp[i, i + n] for i in range(n)])
    Db = np.diag(np.concatenate([inv_nu, inv_nu]))
    S = w @ K_xxpp @ sqrtm(Db)
    return Db, np.linalg.inv(S).T


# ----------------------------------------------------------------------------
# Per-cut truncation to chi  (kron_cpu.py:92-127)
# ----------------------------------------------------------------------------
def thermal_photons(nbar: float, cutoff: int = 20) -> np.ndarray:
    """Geometric photon-number distribution of a thermal mode (kron_cpu.py:92-93)."""
    return 1.0 / (nbar + 1.0) * (nbar / (nbar + 1.0)) ** np.arange(cutoff)


def get_cumsum_kron(sq_cov: np.ndarray, L: int, chi: int = 100, max_dim: int = 10 ** 5,
                    cutoff: int = 6, err_tol: float = 1e-12):
    """Schmidt weights ``res`` (descending), Fock labels ``num`` and Williamson
    symplectic ``S`` of the cut between modes < L and modes >= L
    (kron_cpu.py:95-127, FP64: the float16 cast of ``res`` is dropped).

    Each step multiplies the kept products by the next mode's thermal
    distribution, drops weights <= err_tol, keeps the max_dim largest and
    extends the labels by the new mode's photon number; finally the chi
    largest are returned in descending order.
    """
    M = sq_cov.shape[0] // 2
    sel = np.concatenate([np.arange(L, M), np.arange(L, M) + M])
    D, S = williamson(sq_cov[np.ix_(sel, sel)])
    nbar = (np.diag(D) - 1.0) / 2.0
    nbar[nbar < 0] = 0.0
    res = thermal_photons(nbar[0], cutoff)
    num = np.arange(cutoff, dtype=np.int8)
    for mode in range(1, M - L):
        prod = np.outer(res, thermal_photons(nbar[mode], cutoff)).reshape(-1)
        alive = np.nonzero(prod > err_tol)[0]
        prod = prod[alive]
        top = np.argsort(prod)[-min(len(prod), max_dim):]
        res = prod[top][::-1]
        parents = alive[top][::-1]
        if num.ndim == 1:
            num = num.reshape(-1, 1)
        digits = np.arange(cutoff).reshape(-1, 1)[parents % cutoff]
        num = np.concatenate([num[parents // cutoff], digits], axis=1)
    k = min(chi, len(res))
    top = np.argsort(res)[-k:]
    top = top[np.argsort(res[top])]
    return res[top][::-1], num[top][::-1].astype(np.int8), S


def run_kron(sq_cov: np.ndarray, d: int, chi: int, max_dim: int = 10 ** 5) -> List[tuple]:
    """All M-1 cuts, as kron_cpu.py:147-153 writes them (list of (res, num, S))."""
    M = sq_cov.shape[0] // 2
    return [get_cumsum_kron(sq_cov, c + 1, chi=chi, max_dim=max_dim, cutoff=d) for c in range(M - 1)]


# ----------------------------------------------------------------------------
# Index bookkeeping  (MPS_cpu.py:19-47, 314-332)
# ----------------------------------------------------------------------------
def get_target(num: np.ndarray) -> np.ndarray:
    """Expand Fock labels to repeated 1-based mode indices, left-aligned and
    zero-padded to the largest row sum (MPS_cpu.py:314-332)."""
    num = np.asarray(num)
    rows, modes = num.shape
    width = int(num.sum(axis=1).max()) if rows else 0
    out = np.zeros((rows, width), dtype=np.int32)
    for r in range(rows):
        idx = np.repeat(np.arange(1, modes + 1, dtype=np.int32), num[r].astype(np.int64))
        out[r, : len(idx)] = idx
    return out


def push_to_end(target: np.ndarray) -> np.ndarray:
    """Right-align the non-zero entries of each row, keeping their order
    (MPS_cpu.py:39-47)."""
    out = np.zeros_like(target)
    for r in range(target.shape[0]):
        nz = target[r][target[r] != 0]
        if len(nz):
            out[r, -len(nz):] = nz
    return out


def Sigma_select(Sigma: np.ndarray, target: np.ndarray) -> np.ndarray:
    """Batched gather Sigma2[b] = Sigma[t_b][:, t_b] (MPS_cpu.py:19-37,
    direct_mps_kernels.cu:3-39)."""
    t = np.asarray(target, dtype=np.int64)
    return Sigma[t[:, :, None], t[:, None, :]].astype(CDT)


# ----------------------------------------------------------------------------
# Batched hafnian  (MPS_cpu.py:117-187)
# ----------------------------------------------------------------------------
def hafnian(A: np.ndarray) -> np.ndarray:
    """Hafnians of a batch [B, n, n] of symmetric matrices (MPS_cpu.py:117-140):
    n = 0 -> 1, odd n -> 0, n = 2 and 4 in closed form, else the polynomial
    recursion."""
    B, n, _ = A.shape
    if n == 0:
        return np.ones(B, dtype=CDT)
    if n % 2:
        return np.zeros(B, dtype=CDT)
    if n == 2:
        return A[:, 0, 1].astype(CDT)
    if n == 4:
        return (A[:, 0, 1] * A[:, 2, 3] + A[:, 0, 2] * A[:, 1, 3] + A[:, 0, 3] * A[:, 1, 2]).astype(CDT)
    return recursive_hafnian(A)


def _tri(j: int, k: int) -> int:
    """Packed index of the vertex pair (j, k), j > k."""
    return j * (j - 1) // 2 + k


def recursive_hafnian(A: np.ndarray) -> np.ndarray:
    """Set up the pair polynomials for the recursion (MPS_cpu.py:143-160).

    Row ``_tri(j, k)`` of ``z`` holds the polynomial (in x, truncated at degree
    n/2) attached to the vertex pair (j, k); initially the constant A[j, k].
    ``g`` is the running product polynomial, initially 1.
    """
    B, n2, m2 = A.shape
    if n2 != m2:
        raise ValueError("Matrix must be square")
    if n2 % 2:
        raise ValueError("Matrix size must be even")
    h = n2 // 2
    z = np.zeros((B, h * (2 * h - 1), h + 1), dtype=A.dtype)
    for j in range(1, n2):
        for k in range(j):
            z[:, _tri(j, k), 0] = A[:, j, k]
    g = np.zeros((B, h + 1), dtype=A.dtype)
    g[:, 0] = 1
    return _solve(z, n2, 1, g, h)


def _solve(b: np.ndarray, s: int, w: int, g: np.ndarray, h: int) -> np.ndarray:
    """One level of the recursion on ``s`` vertices (MPS_cpu.py:163-187).

    Vertices 0 and 1 are eliminated.  Branch one drops them (sign flips);
    branch two multiplies g by (1 + x * b01) and adds
    x * (b_{j0} b_{k1} + b_{k0} b_{j1}) to every remaining pair (j, k).
    At s = 0 the result is w * g[h].
    """
    if s == 0:
        return w * g[:, h]
    B = b.shape[0]
    rest = s - 2
    c = np.zeros((B, rest * (rest - 1) // 2, h + 1), dtype=g.dtype)
    for j in range(1, rest):
        for k in range(j):
            c[:, _tri(j, k)] = b[:, _tri(j + 2, k + 2)]
    drop = _solve(c, rest, -w, g, h)
    e = g.copy()
    b01 = b[:, _tri(1, 0)]
    for u in range(h):
        for v in range(h - u):
            e[:, u + v + 1] += g[:, u] * b01[:, v]
    for j in range(1, rest):
        bj0 = b[:, _tri(j + 2, 0)]
        bj1 = b[:, _tri(j + 2, 1)]
        for k in range(j):
            bk0 = b[:, _tri(k + 2, 0)]
            bk1 = b[:, _tri(k + 2, 1)]
            row = _tri(j, k)
            for u in range(h):
                for v in range(h - u):
                    c[:, row, u + v + 1] += bj0[:, u] * bk1[:, v] + bk0[:, u] * bj1[:, v]
    return drop + _solve(c, rest, w, e, h)


def hafnian_bruteforce(A: np.ndarray) -> complex:
    """Sum over perfect matchings (independent check for small n)."""
    n = A.shape[0]
    if n == 0:
        return 1.0 + 0j
    if n % 2:
        return 0j

    def rec(verts):
        if not verts:
            return 1.0 + 0j
        a = verts[0]
        tot = 0j
        for i in range(1, len(verts)):
            b = verts[i]
            tot += A[a, b] * rec(verts[1:i] + verts[i + 1:])
        return tot

    return rec(list(range(n)))


# ----------------------------------------------------------------------------
# Sigma of a site  (MPS_cpu.py:189-229, 305-312, 357-372)
# ----------------------------------------------------------------------------
def blochmessiah(S: np.ndarray):
    """Bloch-Messiah S = O1 D O2 by polar decomposition and a Takagi
    factorisation of the squeezing block (MPS_cpu.py:189-229)."""
    N = S.shape[0]
    h = N // 2
    I = np.eye(h)
    R = np.block([[I, 1j * I], [I, -1j * I]]) / np.sqrt(2)
    Sc = R @ S @ R.conj().T
    u1, d1, v1 = svd(Sc, lapack_driver="gesvd")
    herm = u1 @ np.diag(d1) @ u1.conj().T
    unit = u1 @ v1
    alpha = unit[:h, :h]
    beta = herm[:h, h:]
    u2, d2, v2 = np.linalg.svd(beta)
    sval = np.arcsinh(d2)
    tak = u2 @ sqrtm(u2.conj().T @ v2.T)
    Z = 0 * tak
    uf = np.block([[tak, Z], [Z, tak.conj()]])
    left = tak.conj().T @ alpha
    vf = np.block([[left, Z], [Z, left.conj()]])
    df = np.block([[np.diag(np.cosh(sval)), np.diag(np.sinh(sval))],
                   [np.diag(np.sinh(sval)), np.diag(np.cosh(sval))]])
    back = lambda X: np.real_if_close(R.conj().T @ X @ R)
    return back(uf), back(df), back(vf)


def get_U2_sq_U1(S_l: np.ndarray, S_r: np.ndarray):
    """Passive unitaries and squeezing of (1 (+) S_l)^-1 S_r (MPS_cpu.py:357-372)."""
    M = S_r.shape[0] // 2
    inner = np.concatenate([np.arange(1, M), np.arange(1, M) + M])
    left_inv = np.eye(2 * M)
    left_inv[np.ix_(inner, inner)] = np.linalg.inv(S_l)
    S2, SQ, S1 = blochmessiah(left_inv @ S_r)
    U2 = S2[:M, :M] - 1j * S2[:M, M:]
    U1 = S1[:M, :M] - 1j * S1[:M, M:]
    sq = np.log(np.diag(SQ)[:M])
    return U2, sq, U1


def get_Sigma(U2: np.ndarray, sq: np.ndarray, U1: np.ndarray) -> np.ndarray:
    """Fock-amplitude generating matrix of the site's Gaussian unitary
    (MPS_cpu.py:305-312)."""
    M = len(sq)
    th = np.diag(np.tanh(sq))
    sech = np.diag(1.0 / np.cosh(sq))
    Sigma = np.zeros((2 * M, 2 * M), dtype=CDT)
    Sigma[:M, :M] = U2 @ th @ U2.T
    Sigma[:M, M:] = U2 @ sech @ U1
    Sigma[M:, :M] = U1.T @ sech @ U2.T
    Sigma[M:, M:] = -U1.T @ th @ U1
    return Sigma


def A_elem(Sigma: np.ndarray, target: np.ndarray, denominator: np.ndarray,
           max_memory_in_gb: float = 0.5):
    """Amplitudes hafnian(Sigma[t][:, t]) / denominator, chunked by a memory
    budget, with gather and hafnian wall times (MPS_cpu.py:334-355)."""
    B, n = target.shape
    per = max(1, int(max_memory_in_gb * 1e9 // (n * n * 16))) if n else max(B, 1)
    out = np.zeros(B, dtype=CDT)
    t_sel = t_haf = 0.0
    for lo in range(0, B, per):
        hi = min(B, lo + per)
        t0 = time.time()
        sub = Sigma_select(Sigma, target[lo:hi])
        t1 = time.time()
        out[lo:hi] = hafnian(sub)
        t2 = time.time()
        t_sel += t1 - t0
        t_haf += t2 - t1
    return out / denominator, t_haf, t_sel


# ----------------------------------------------------------------------------
# Per-site Gamma build  (MPS_cpu.py:377-525)
# ----------------------------------------------------------------------------
def _log_fact_rows(num: np.ndarray) -> np.ndarray:
    """sqrt(prod_i num_i!) per label row (MPS_cpu.py:413, 437, 468, 479)."""
    return np.sqrt(np.prod(factorial(num.astype(np.float64)), axis=1))


def build_site(site: int, M: int, d: int, chi: int, sq_cov: np.ndarray, cuts: Sequence[tuple],
               err_tol: float = 1e-10, S_full: Optional[np.ndarray] = None,
               stats: Optional[Dict] = None):
    """Gamma_site [chi, chi, d] and Lambda_site [chi] (None for the last site),
    following the three branches of MPS_cpu.py:402-520.

    ``cuts[c] = (res_c, num_c, S_c)`` is kron's output for cut c (between
    modes c and c+1).  Axis 0 of Gamma is the bond of cut site-1 (the
    reference's "right"/"pre" labels), axis 1 the bond of cut ``site``.
    """
    Gamma = np.zeros((chi, chi, d), dtype=CDT)
    Lam = np.zeros(chi, dtype=np.float64)
    if stats is None:
        stats = {}
    stats.setdefault("items", 0)
    stats.setdefault("haf_s", 0.0)

    if site == 0:
        if S_full is None:
            S_full = williamson(sq_cov)[1]
        res, num, S_l = cuts[0]
        keep = res > err_tol
        num = num[keep].reshape(int(keep.sum()), -1)
        res = res[keep]
        U2, sq, U1 = get_U2_sq_U1(S_l, S_full)
        Sigma = get_Sigma(U2, sq, U1)
        lt = get_target(num)
        lsum = num.sum(axis=1)
        lden = _log_fact_rows(num)
        Z = np.sqrt(np.prod(np.cosh(sq)))
        Lam[: len(res)] = np.sqrt(res)
        for j in range(d):
            for size in range(int(lsum.max()) + 1):
                li = np.nonzero(lsum == size)[0]
                if len(li) == 0 or np.all(Lam[li] <= err_tol):
                    continue
                tgt = np.concatenate([np.zeros((len(li), j), np.int32), lt[:, :size][li]], axis=1)
                den = np.sqrt(factorial(j)) * lden[li]
                amp, th, _ = A_elem(Sigma, tgt, den)
                stats["items"] += len(li)
                stats["haf_s"] += th
                Gamma[0, li, j] = amp / Z / Lam[li]
        return Gamma, Lam

    if site == M - 1:
        _, num_pre, S_r = cuts[site - 1]
        num_pre = num_pre.reshape(num_pre.shape[0], -1)
        rt = get_target(num_pre)
        rsum = num_pre.sum(axis=1)
        rden = _log_fact_rows(num_pre)
        U2, sq, U1 = get_U2_sq_U1(np.zeros((0, 0)), S_r)
        Z = np.sqrt(np.prod(np.cosh(sq)))
        Sigma = get_Sigma(U2, sq, U1)
        for j in range(d):
            for size in range(int(rsum.max()) + 1):
                ri = np.nonzero(rsum == size)[0]
                if j == 0 and size == 0:
                    Gamma[ri, 0, 0] = 1.0 / Z
                    continue
                if len(ri) == 0:
                    continue
                tgt = np.concatenate([np.zeros((len(ri), j), np.int32), rt[:, :size][ri]], axis=1)
                den = np.sqrt(factorial(j)) * rden[ri]
                amp, th, _ = A_elem(Sigma, tgt, den)
                stats["items"] += len(ri)
                stats["haf_s"] += th
                Gamma[ri, 0, j] = amp / Z
        return Gamma, None

    _, num_pre, S_r = cuts[site - 1]
    num_pre = num_pre.reshape(num_pre.shape[0], -1)
    rt = push_to_end(get_target(num_pre))
    rsum = num_pre.sum(axis=1)
    rden = _log_fact_rows(num_pre)
    res, num, S_l = cuts[site]
    keep = res > err_tol
    num = num[keep].reshape(int(keep.sum()), -1)
    res = res[keep]
    lt = get_target(num)
    lw = lt.shape[1]
    lsum = num.sum(axis=1)
    full = lsum[:, None] + rsum[None, :]
    lden = _log_fact_rows(num)
    U2, sq, U1 = get_U2_sq_U1(S_l, S_r)
    Sigma = get_Sigma(U2, sq, U1)
    Z = np.sqrt(np.prod(np.cosh(sq)))
    Lam[: len(res)] = np.sqrt(res)
    m_l = num.shape[1]
    for j in range(d):
        for size in range(int(full.max()) + 1):
            li, ri = np.nonzero(full == size)
            if len(li) == 0 or np.all(Lam[li] <= err_tol):
                continue
            if j == 0 and size == 0:
                Gamma[ri, li, 0] = 1.0 / Z / Lam[li]
                continue
            tgt = np.zeros((len(li), size), np.int32)
            left = lt[:, :size][li]
            tgt[:, : min(lw, size)] = left
            if size:
                right = rt[:, -size:][ri].copy()
                right[right != 0] += m_l
                tgt[:, -right.shape[1]:] += right
            tgt = np.concatenate([np.zeros((len(li), j), np.int32), tgt], axis=1)
            den = np.sqrt(factorial(j)) * lden[li] * rden[ri]
            amp, th, _ = A_elem(Sigma, tgt, den)
            stats["items"] += len(li)
            stats["haf_s"] += th
            Gamma[ri, li, j] = amp / Z / Lam[li]
    return Gamma, Lam


def build_mps(sq_cov: np.ndarray, d: int, chi: int, cuts: Sequence[tuple],
              sites: Optional[Sequence[int]] = None, err_tol: float = 1e-10):
    """Run the site loop of MPS_cpu.py:384-525 (optionally a subset of sites)."""
    M = sq_cov.shape[0] // 2
    S_full = williamson(sq_cov)[1]
    out = {}
    for s in (range(M) if sites is None else sites):
        out[s] = build_site(s, M, d, chi, sq_cov, cuts, err_tol=err_tol, S_full=S_full)
    return out


# ----------------------------------------------------------------------------
# Consumers of Gamma/Lambda: pattern probabilities and the sampler
# ----------------------------------------------------------------------------
def pattern_amplitudes(Gammas: Sequence[np.ndarray], Lambdas: Sequence[np.ndarray],
                       patterns: np.ndarray) -> np.ndarray:
    """Amplitude of each photon pattern n_0..n_{M-1} of the MPS state:
    v <- (v * Lambda_{i-1}) @ Gamma_i[:, :, n_i] from site 0 (row 0 of
    Gamma_0) to site M-1 (column 0), the transfer step of sampling_cpu.py:75-80
    with the photon numbers fixed instead of drawn."""
    P, M = patterns.shape
    v = Gammas[0][0][:, patterns[:, 0]].T.astype(CDT)  # [P, chi]
    for i in range(1, M):
        v = v * Lambdas[i - 1][None, :]
        G = Gammas[i]
        nxt = np.zeros((P, G.shape[1]), dtype=CDT)
        for n in np.unique(patterns[:, i]):
            sel = patterns[:, i] == n
            nxt[sel] = v[sel] @ G[:, :, n]
        v = nxt
    return v[:, 0]


def enumerate_patterns(M: int, max_total: int, d: int) -> np.ndarray:
    """All patterns with at most ``max_total`` photons and <= d-1 per mode,
    ordered by total photon number then lexicographically."""
    out = [np.zeros(M, dtype=np.int32)]

    def rec(start, left, cur):
        for m in range(start, M):
            for c in range(1, min(left, d - 1) + 1):
                cur[m] += c
                out.append(cur.copy())
                if left - c > 0:
                    rec(m + 1, left - c, cur)
                cur[m] -= c

    rec(0, max_total, np.zeros(M, dtype=np.int32))
    pats = np.array(out, dtype=np.int32)
    tot = pats.sum(axis=1)
    order = np.lexsort(tuple(pats[:, ::-1].T) + (tot,))
    return pats[order]


def _destroy(n: int) -> np.ndarray:
    return np.diag(np.sqrt(np.arange(1, n, dtype=CDT)), 1)


def batch_displaces(dd: int, alphas: np.ndarray) -> np.ndarray:
    """D(alpha) = expm(alpha a^dag - alpha^* a) per sample and mode, shape
    [n, M, dd, dd] (sampling_cpu.py:133-148)."""
    a = _destroy(dd)
    ad = a.conj().T
    n, M = alphas.shape
    out = np.zeros((n, M, dd, dd), dtype=CDT)
    for m in range(M):
        al = alphas[:, m].reshape(-1, 1, 1)
        out[:, m] = expm(al * ad[None] - np.conj(al) * a[None])
    return out


def sample(Gammas: Sequence[np.ndarray], Lambda: np.ndarray, sqrtW: np.ndarray, dd: int,
           n: int, rng: np.random.RandomState) -> np.ndarray:
    """Photon-number samples of the lossy state: random displacement drawn
    from the thermal part, then sequential inverse-CDF sampling along the
    chain (sampling_cpu.py:30-117).  ``Lambda`` is [chi, M-1]."""
    M = sqrtW.shape[0] // 2
    chi = Gammas[0].shape[0]
    d = Gammas[0].shape[2]
    mu = (sqrtW @ rng.normal(size=(2 * M, n))).T
    alpha = (mu[:, :M] + 1j * mu[:, M:]) / np.sqrt(4.0)
    D = batch_displaces(dd, alpha)
    out = []
    pre = None
    for i in range(M):
        G = np.zeros((chi, chi, dd), dtype=CDT)
        G[:, :, :d] = Gammas[i]
        if i == 0:
            thr = rng.rand(n, 1)
            t = np.einsum("mj,Bkj->Bmk", G.sum(axis=0), D[:, i])
            pre = t.copy()
            p = np.einsum("Bmk,m->Bk", np.abs(t) ** 2, Lambda[:, 0] ** 2)
        else:
            t = (pre * Lambda[:, i - 1]) @ G.reshape(chi, chi * dd)
            t = np.einsum("Bmj,Bkj->Bmk", t.reshape(n, chi, dd), D[:, i])
            pre = t.copy()
            if i == M - 1:
                p = np.abs(t[:, 0, :]) ** 2
            else:
                p = np.einsum("Bmk,m->Bk", np.abs(t) ** 2, Lambda[:, i] ** 2)
            thr = rng.rand(n, 1)
        p = p / p.sum(axis=1, keepdims=True)
        k = (thr > np.cumsum(p, axis=1)).sum(axis=1)
        out.append(k)
        if i == M - 1:
            break
        pre = pre[np.arange(n), :, k]
    return np.array(out).T
