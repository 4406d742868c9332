"""Seeded synthetic inputs for the tSVD workloads (no external datasets).

``power_law_sectors`` builds U(1) block matrices like the CTM enlarged
corners the projector SVD sees: a seeded number of sectors, square blocks of
log-uniform size, and within each block A_q = U_q diag(s_q) V_q^T with Haar
U_q, V_q and a power-law spectrum s_{q,i} = c_q (i+1)^-alpha."""
from __future__ import annotations

import numpy as np


def haar_orthogonal(rng: np.random.Generator, n: int) -> np.ndarray:
    """Haar-distributed orthogonal matrix: QR of a Gaussian matrix with the
    signs of R's diagonal moved into Q."""
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.where(np.diag(r) == 0, 1.0, np.diag(r)))


def power_law_sectors(seed: int, n_sectors=(9, 15), size=(16, 1024), alphas=(1.0, 2.0, 3.0), scale=(0.1, 1.0),
                      exponent_scale: float = 1.0):
    """Returns a list of (q, n, alpha, c, block) with charges q centred on 0.
    ``exponent_scale`` multiplies every exponent (same sizes, U_q, V_q and c_q
    for a given seed): a sequence of seeds-fixed matrices whose spectra drift,
    like the projector matrices of consecutive CTM steps."""
    rng = np.random.default_rng(seed)
    ns = int(rng.integers(n_sectors[0], n_sectors[1] + 1))
    lo, hi = np.log(size[0]), np.log(size[1])
    out = []
    for a in range(ns):
        q = a - ns // 2
        n = int(round(np.exp(rng.uniform(lo, hi))))
        alpha = float(rng.choice(alphas))
        c = float(rng.uniform(*scale))
        s = c * np.arange(1, n + 1, dtype=np.float64) ** -(alpha * exponent_scale)
        U = haar_orthogonal(rng, n)
        V = haar_orthogonal(rng, n)
        out.append((q, n, alpha, c, (U * s) @ V.T))
    return out


def power_law_spectra(secs, exponent_scale: float = 1.0):
    """The exact singular values (descending) of each block of
    ``power_law_sectors(..., exponent_scale)``."""
    return [c * np.arange(1, n + 1, dtype=np.float64) ** -(alpha * exponent_scale) for _q, n, alpha, c, _b in secs]
