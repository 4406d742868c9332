"""Randomized blockwise tSVD restated in numpy (test infrastructure only).

The randomized form has no counterpart in the reference; its contract is
the reference's Tensor::tSVD (src/Core/Tensor.cpp:478-633): the same
truncation (cutoff_matrices, Tensor.cpp:523-633) applied to per-sector
spectra that come from a sketch instead of a full SVD.  This module follows
the device algorithm step by step so both can be compared on the same
seeded test matrices:

  Omega_i = N(0,1) from (seed, stream i)          n_i x l_i
  Q = orth(A Omega)                               shifted CholeskyQR3
  repeat p times: Q = orth(A orth(A^T Q))
  B = Q^T A = U_B S V^T ,  U = Q U_B ,  sign convention of fix_svd_signs

A sector is decomposed exactly if l_i <= 0 or 2 l_i >= min(m_i, n_i); a
sketched sector that keeps all l_i of its values is redone with 2 l_i
columns (the same Gaussian stream, extended), exactly after the third
doubling.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .basis import Qbasis
from .tensor import Tensor, cutoff_matrices, fix_svd_signs



MAX_RETRIES = 3


def _mix64(z):
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def gaussian(seed: int, stream: int, count: int) -> np.ndarray:
    """Counter-based N(0,1) numbers: Box-Muller on hashed uniforms
    u1 = ((h1 >> 11) + 1) 2^-53 in (0, 1], u2 = (h2 >> 11) 2^-53."""
    base = _mix64(np.uint64(seed) ^ _mix64(np.array([stream], dtype=np.uint64)))[0]
    e = np.arange(count, dtype=np.uint64)
    h1 = _mix64(base ^ (np.uint64(2) * e))
    h2 = _mix64(base ^ (np.uint64(2) * e + np.uint64(1)))
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53
    u2 = (h2 >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def _chol_pass(Y, shift):
    """One CholeskyQR pass: Y R^-1 with R^T R = Y^T Y + shift * (m l + l (l + 1)) tr(Y^T Y) I.
    A pivot that is not above f = max(eps tr(Y^T Y) / l, 1e-300) (an exactly or
    numerically rank-deficient Y) becomes sqrt(f) with the rest of its column
    zeroed, so the factor stays finite and the direction is dropped."""
    m, l = Y.shape
    G = Y.T @ Y
    tr = np.trace(G)
    s = shift * (m * l + l * (l + 1)) * tr
    floor = max(np.finfo(float).eps * (tr / l if tr > 0 else 0.0), 1e-300)
    L = np.zeros((l, l))
    for j in range(l):
        d = G[j, j] + s - L[j, :j] @ L[j, :j]
        if d > floor:
            L[j, j] = np.sqrt(d)
            L[j + 1:, j] = (G[j + 1:, j] - L[j + 1:, :j] @ L[j, :j]) / L[j, j]
        else:
            L[j, j] = np.sqrt(floor)
    return sla.solve_triangular(L, Y.T, lower=True).T  # Y L^-T


# CholeskyQR passes of the bases between the products of a subspace iteration
INTER_PASSES = 1


def _orth(Y, passes=3):
    """Shifted CholeskyQR3 (Fukaya et al., SIAM J. Sci. Comput. 2020), as on
    the device: one pass with shift 11 u, then up to two plain passes
    (``passes`` in 1..3)."""
    if Y.size == 0:
        return Y.copy()
    Q = _chol_pass(Y, 11.0 * 2.0 ** -53)
    for _ in range(passes - 1):
        Q = _chol_pass(Q, 0.0)
    return Q


def sketch_svd(A, l, power_iters, seed, stream, warm_rows=None):
    """Rank-l randomized SVD of one block (U m x l, s l, Vt l x n), sign-fixed.
    ``warm_rows`` (k x n, optional): its first min(k, l) rows replace the first
    Gaussian columns of Omega."""
    m, n = A.shape
    Om = gaussian(seed, stream, n * l).reshape((n, l), order="F")
    if warm_rows is not None and warm_rows.shape[1] == n:
        kw = min(warm_rows.shape[0], l)
        Om[:, :kw] = warm_rows[:kw, :].T
    Q = _orth(A @ Om, INTER_PASSES if power_iters > 0 else 3)
    for it in range(power_iters):
        Q = _orth(A @ _orth(A.T @ Q, INTER_PASSES), 3 if it + 1 == power_iters else INTER_PASSES)
    ub, s, vt = np.linalg.svd(Q.T @ A, full_matrices=False)
    u, vt = fix_svd_signs(Q @ ub, vt)
    return u, s, vt


def tsvd_randomized(T: Tensor, max_keep, eps_svd, sketch, power_iters=1, seed=0, warm=None):
    """Returns (U, S, Vdag, truncWeight, entropy, keep, width, n_saturated).
    ``warm``: optional V^dag tensor of an earlier decomposition (same column
    bases) seeding the sketches."""
    n = len(T.sectors)
    assert len(sketch) == n
    exact = [False] * n
    want = [int(x) for x in sketch]
    saturated = 0
    for rnd in range(MAX_RETRIES + 1):
        width = []
        for i, b in enumerate(T.blocks):
            kmin = min(b.shape)
            l = want[i]
            if exact[i] or l <= 0 or 2 * l >= kmin:
                exact[i] = True
                l = kmin
            width.append(l)
        sym = T.sym
        middle = Qbasis(sym, 1)
        for q, l in zip(T.sectors, width):
            middle.push_back(q, l)
        U = Tensor(sym, T.dom, [middle], fill=False)
        S = Tensor(sym, [middle], [middle], fill=False)
        Vd = Tensor(sym, [middle], T.cod, fill=False)
        allsv = []
        for i, (q, b) in enumerate(zip(T.sectors, T.blocks)):
            if exact[i]:
                u, s, vt = sla.svd(b, full_matrices=False, lapack_driver="gesvd")
                u, vt = fix_svd_signs(u, vt)
            else:
                wr = warm.block(q) if warm is not None and warm.has(q) else None
                u, s, vt = sketch_svd(b, width[i], power_iters, seed, i, wr)
            allsv.extend((q, float(v)) for v in s)
            U.push_back(q, u)
            S.push_back(q, np.diag(s))
            Vd.push_back(q, vt)
        oU, oS, oV, tw, ent = cutoff_matrices(T, U, S, Vd, allsv, max_keep, eps_svd, False, False)
        keep = [oS.block(q).shape[0] if q in oS._dict else 0 for q in T.sectors]
        sat = [i for i in range(n) if not exact[i] and keep[i] >= width[i]]
        if not sat:
            return oU, oS, oV, tw, ent, keep, width, saturated
        for i in sat:
            want[i] = 2 * width[i]
            if rnd + 1 >= MAX_RETRIES:
                exact[i] = True
        saturated += len(sat)
