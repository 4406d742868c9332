"""CPU emulation of the tensor-core sketch products of the randomized tSVD.

The device runs the first product A Omega and both products of the leading
subspace iterations as 3xTF32 tensor-core GEMMs. The pack kernel splits every
FP64 operand x into hi = tf32(float(x)) and lo = tf32(float(x - hi)), rounding to
nearest with ties away from zero, and accumulates hi*hi + hi*lo + lo*hi in FP32.
The last `tail` iterations, the final CholeskyQR3 and the projection stay FP64.
Emulated here with numpy on graded power-law blocks (the shape of the CTM
projector spectra): with two FP64 iterations at the end, the singular values
and the kept subspace of the all-FP64 sketch come back to FP64-level accuracy.
"""
import numpy as np

from oracle.rsvd import _orth, gaussian
from xped_gb300.workloads import power_law_sectors


def _tf32(x32):
    b = x32.view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def _split(x):
    hi = _tf32(x.astype(np.float32))
    lo = _tf32((x - hi.astype(np.float64)).astype(np.float32))
    return hi, lo


def _mm3(A, X):
    Ah, Al = _split(A)
    Xh, Xl = _split(X)
    return (Ah @ Xh + Ah @ Xl + Al @ Xh).astype(np.float64)


def _sketch(A, l, iters, seed, stream, tail):
    """Device order of tsvd_randomized: tc_iters = iters - tail leading
    iterations (and A Omega) in emulated 3xTF32, the rest FP64."""
    tc = max(0, iters - tail) if tail >= 0 else 0
    n = A.shape[1]
    Om = gaussian(seed, stream, n * l).reshape((n, l), order="F")
    mul = lambda M, X, low: _mm3(M, X) if low else M @ X
    Q = _orth(mul(A, Om, tc > 0), 1)
    for p in range(iters):
        Z = _orth(mul(A.T, Q, p < tc), 1)
        Q = _orth(mul(A, Z, p < tc), 3 if p + 1 == iters else 1)
    u, s, vt = np.linalg.svd(Q.T @ A, full_matrices=False)
    return Q @ u, s


def test_split_products_are_fp32_accurate():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((200, 300))
    X = rng.standard_normal((300, 24))
    ref = A @ X
    err = np.abs(_mm3(A, X) - ref).max() / np.abs(ref).max()
    assert 1e-10 < err < 1e-5  # visibly not FP64, about FP32 accumulation


def _worst(tail):
    """Largest kept-sigma difference (relative to sigma_max) and largest
    difference of the kept-subspace projectors against the all-FP64 sketch."""
    worst_s = worst_u = 0.0
    checked = 0
    for q, n, _alpha, _c, b in power_law_sectors(3, n_sectors=(9, 11), size=(72, 384)):
        l = min(40, n // 3)  # >= 24: at least 8 kept columns below the 16 of oversampling
        u0, s0 = _sketch(b, l, 8, 5, q + 100, -1)
        u1, s1 = _sketch(b, l, 8, 5, q + 100, tail)
        k = l - 16
        worst_s = max(worst_s, np.abs(s1[:k] - s0[:k]).max() / s0[0])
        worst_u = max(worst_u, np.abs(u0[:, :k] @ u0[:, :k].T - u1[:, :k] @ u1[:, :k].T).max())
        checked += 1
    assert checked >= 8
    return worst_s, worst_u


def test_two_fp64_iterations_restore_the_fp64_sketch():
    s2, u2 = _worst(2)
    s0, u0 = _worst(0)
    print("tail 2: sigma diff", s2, "subspace diff", u2, "| all products 3xTF32:", s0, u0)
    assert s2 < 1e-13 and u2 < 1e-7
    # without the FP64 tail the kept subspace stays at the products' FP32-level error
    assert u0 > 100 * u2
