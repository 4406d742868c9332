"""The reference's reverse-mode checks for `operator*`, `permute` and `tSVD`
(tests/ad.cpp:230-388,507-592 with tests/ad_tests.hpp:10-33: the AD gradient of a
scalar function of a random `Tensor<2,2>` equals its finite-difference
gradient over the stored entries), restated for the oracle's reverse rules,
which the device's `matmul_backward` and `permute_adj` are compared against:

* f(t) = <G, t * c> with c fixed: df/dt = G * c^dagger  (ADTensor.hpp:741-752);
* f(t) = <G, t * t>: df/dt = G * t^dagger + t^dagger * G (both operands depend on t);
* f(t) = <G, t.permute<shift>(p)>: df/dt = G.permute_adj<shift>(p)  (ADTensor.hpp:172-184);
* weighted singular values and <G, U V^dagger> through the full tSVD: the per-sector SVD reverse
  rule (ADTensor.hpp:257-301), by central differences with a small step.

<.,.> is the sum over stored entries, as the reference's finite differences
perturb stored entries.  The product and permute functions are linear (or
quadratic) in each entry, so central differences with a unit step are exact up
to rounding."""
import itertools

import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from helpers import random_pairs


def _random_t22(rng, symname, size):
    s = oracle.make_symmetry(symname)
    B1 = Qbasis.from_pairs(s, random_pairs(rng, symname, size), sort=True)
    B2 = Qbasis.from_pairs(s, random_pairs(rng, symname, size), sort=True)
    return s, oracle.Tensor(s, [B1, B2], [B1, B2]).set_random(rng)


def _with_data(t, x):
    out = t.copy()
    k = 0
    for i, b in enumerate(out.blocks):
        out.blocks[i] = x[k:k + b.size].reshape(b.shape, order="F").copy()
        k += b.size
    return out


def _fd_gradient(f, t):
    x0 = t.data()
    g = np.zeros_like(x0)
    for i in range(x0.size):
        e = np.zeros_like(x0)
        e[i] = 1.0
        g[i] = (f(_with_data(t, x0 + e)) - f(_with_data(t, x0 - e))) / 2.0
    return g


def _aligned(grad, like):
    """`grad`'s blocks in `like`'s sector order (zero where grad has no block)."""
    return np.concatenate([(grad.block(q) if grad.has(q) else np.zeros_like(b)).ravel(order="F")
                           for q, b in zip(like.sectors, like.blocks)]) if like.blocks else np.zeros(0)


SIZES = {"u1": 5, "fz2": 5, "su2": 6}


@pytest.mark.parametrize("symname", ["u1", "fz2", "su2"])
def test_matmul_reverse_rule_matches_finite_differences(symname):
    rng = np.random.default_rng(21)
    s, t = _random_t22(rng, symname, SIZES[symname])
    c = oracle.Tensor(s, t.cod, t.cod).set_random(rng)
    G = oracle.Tensor(s, t.dom, t.cod).set_random(rng)

    def inner(a, b):
        return sum(float((a.block(q) * b.block(q)).sum()) for q in a.sectors if b.has(q))

    fd = _fd_gradient(lambda x: inner(G, x * c), t)
    assert np.abs(fd - _aligned(G * c.adjoint(), t)).max() <= 1e-10 * max(1.0, np.abs(fd).max())
    fd2 = _fd_gradient(lambda x: inner(G, x * x), t)
    rule2 = _aligned(G * t.adjoint(), t) + _aligned(t.adjoint() * G, t)
    assert np.abs(fd2 - rule2).max() <= 1e-10 * max(1.0, np.abs(fd2).max())


@pytest.mark.parametrize("symname", ["u1", "fz2", "su2"])
def test_permute_reverse_rule_matches_finite_differences(symname):
    rng = np.random.default_rng(22)
    s, t = _random_t22(rng, symname, SIZES[symname])
    for shift, p in [(0, (0, 1, 2, 3)), (0, (1, 0, 3, 2)), (1, (0, 2, 1, 3)), (-1, (3, 1, 0, 2)), (2, (2, 3, 0, 1))]:
        y = t.permute(shift, list(p))
        G = oracle.Tensor(s, y.dom, y.cod).set_random(rng)

        def f(x):
            z = x.permute(shift, list(p))
            return sum(float((G.block(q) * z.block(q)).sum()) for q in z.sectors if G.has(q))

        fd = _fd_gradient(f, t)
        rule = _aligned(G.permute_adj(shift, list(p)), t)
        assert np.abs(fd - rule).max() <= 1e-10 * max(1.0, np.abs(fd).max()), (shift, p)


@pytest.mark.parametrize("symname", ["u1", "fz2", "su2"])
def test_tsvd_reverse_rule_matches_finite_differences(symname):
    """tests/ad.cpp:507-592 (the gauge-invariant cases): a weighted sum of the singular values and
    <G, U V^dagger>, through the full (untruncated) tSVD of a random Tensor<2,2>, against the per-sector
    reverse rule svd_backward_block (ADTensor.hpp:257-301) embedded in the tensor's sectors."""
    from oracle.tensor import svd_backward_block
    rng = np.random.default_rng(23)
    s, t = _random_t22(rng, symname, SIZES[symname])
    big = 10 ** 6

    def parts(x):
        U, S, Vd, _, _ = x.tsvd(big, 0.0)
        return U, S, Vd

    U0, S0, V0 = parts(t)
    g = {q: rng.standard_normal(S0.block(q).shape[0]) for q in S0.sectors}
    G = {q: rng.standard_normal((U0.block(q).shape[0], V0.block(q).shape[1])) for q in U0.sectors}

    def f_sigma(x):
        _, S, _ = parts(x)
        return sum(float(g[q] @ np.diag(S.block(q))) for q in S.sectors)

    def f_uv(x):
        U, _, Vd = parts(x)
        return sum(float((G[q] * (U.block(q) @ Vd.block(q))).sum()) for q in U.sectors)

    def fd(f, h=1e-6):
        x0 = t.data()
        out = np.zeros_like(x0)
        for i in range(x0.size):
            e = np.zeros_like(x0)
            e[i] = h
            out[i] = (f(_with_data(t, x0 + e)) - f(_with_data(t, x0 - e))) / (2 * h)
        return out

    def rule(which):
        blocks = []
        for q, b in zip(t.sectors, t.blocks):
            u, sv, vd = U0.block(q), np.diag(S0.block(q)), V0.block(q)
            zu, zs, zv = np.zeros_like(u), np.zeros((sv.size, sv.size)), np.zeros_like(vd)
            if which == "sigma":
                dA = svd_backward_block(u, sv, vd, zu, np.diag(g[q]), zv)
            else:
                dA = svd_backward_block(u, sv, vd, G[q] @ vd.T, zs, u.T @ G[q])
            blocks.append(dA.ravel(order="F"))
        return np.concatenate(blocks)

    for f, which in ((f_sigma, "sigma"), (f_uv, "uv")):
        num, ana = fd(f), rule(which)
        assert np.abs(num - ana).max() <= 1e-6 * max(1.0, np.abs(num).max()), which
