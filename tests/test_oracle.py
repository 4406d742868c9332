"""Pins the CPU oracle to the reference's own test properties (no golden
vectors exist upstream; tests/tensor_tests.hpp, tests/tree_tests.hpp and
tests/ad.cpp assert identities, restated here) plus exact SU(2) 6j values."""
import itertools
from fractions import Fraction

import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis, decompose_permutation, inverse_permutation, treepair_permute
from oracle.sym import wigner6j_twice
from oracle.tensor import get_permutations, decompose
from helpers import random_pairs


def _rand_basis(rng, sym, n, qrange):
    b = Qbasis(sym, 1)
    while b.fullDim() < n:
        q = int(rng.integers(*qrange))
        d = int(rng.integers(1, 3))
        if b.fullDim() + sym.degeneracy(q) * d <= n:
            b.push_back(q, d)
    return b


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_permute_equals_dense_shuffle_u1(seed):
    """tests/tensor_tests.hpp:1-48 over all 24 permutations and shifts -2..2
    (tests/tensor.cpp:188-227), U(1), unsorted random bases of size 5."""
    rng = np.random.default_rng(seed)
    s = oracle.U1()
    B, C = _rand_basis(rng, s, 5, (-3, 4)), _rand_basis(rng, s, 5, (-3, 4))
    t = oracle.Tensor(s, [B, C], [B, C]).set_random(rng)
    P = t.plain_tensor()
    for p in itertools.permutations(range(4)):
        for shift in range(-2, 3):
            tp = t.permute(shift, list(p))
            assert np.array_equal(tp.plain_tensor(), np.transpose(P, p))


def test_permute_within_domain_codomain_rank4():
    """Within-domain permutations of Tensor<4,0> / <0,4> (tensor_tests.hpp:111-303)."""
    rng = np.random.default_rng(9)
    s = oracle.U1()
    Bs = [_rand_basis(rng, s, 4, (-2, 3)) for _ in range(4)]
    t = oracle.Tensor(s, Bs, []).set_random(rng)
    P = t.plain_tensor()
    for p in itertools.permutations(range(4)):
        assert np.array_equal(t.permute(0, list(p)).plain_tensor(), np.transpose(P, p))
    t2 = oracle.Tensor(s, [], Bs).set_random(rng)
    P2 = t2.plain_tensor()
    for p in itertools.permutations(range(4)):
        assert np.array_equal(t2.permute(0, list(p)).plain_tensor(), np.transpose(P2, p))


@pytest.mark.parametrize("symname,pairs", [("fu1", [(-1, 2), (0, 1), (1, 2), (2, 1)]), ("fz2", [(0, 2), (1, 3)]),
                                           ("su2", [(1, 2), (2, 1), (3, 1)])])
def test_permute_round_trip_and_norm(symname, pairs):
    rng = np.random.default_rng(4)
    s = oracle.make_symmetry(symname)
    B = Qbasis.from_pairs(s, pairs, sort=False)
    C = Qbasis.from_pairs(s, pairs[::-1], sort=False)
    t = oracle.Tensor(s, [B, C], [B, C]).set_random(rng)
    for p in itertools.permutations(range(4)):
        for shift in range(-2, 3):
            tp = t.permute(shift, list(p))
            back = tp.permute(-shift, inverse_permutation(p))
            for q in t.sectors:
                assert np.allclose(back.block(q), t.block(q), atol=1e-13)
            assert abs(tp.squared_norm() - t.squared_norm()) < 1e-11 * t.squared_norm()


@pytest.mark.parametrize("symname", ["u1", "fu1", "su2"])
def test_tree_swap_and_permute_round_trips(symname):
    """tests/tree_tests.hpp:1-167: swap(pos) twice and permute(p) then p^-1
    give coefficient 1 on the original tree and 0 elsewhere."""
    s = oracle.make_symmetry(symname)
    if symname == "su2":
        B = Qbasis.from_pairs(s, [(1, 1), (2, 1), (3, 1)])
    else:
        B = Qbasis.from_pairs(s, [(-1, 1), (0, 1), (1, 1)])
    BCDE = B.combine(B).combine(B).combine(B)
    for q in BCDE.qs:
        for tree in BCDE.trees[q]:
            for pos in range(3):
                acc = {}
                for t2, c in tree.swap(s, pos).items():
                    for t3, c2 in t2.swap(s, pos).items():
                        acc[t3] = acc.get(t3, 0.0) + c * c2
                for t3, c in acc.items():
                    assert abs(c - (1.0 if t3 == tree else 0.0)) < 1e-12
            for p in itertools.permutations(range(4)):
                acc = {}
                for t2, c in tree.permute(s, list(p)).items():
                    for t3, c2 in t2.permute(s, inverse_permutation(p)).items():
                        acc[t3] = acc.get(t3, 0.0) + c * c2
                for t3, c in acc.items():
                    assert abs(c - (1.0 if t3 == tree else 0.0)) < 1e-12


def test_treepair_permute_round_trip_su2():
    """treepair::permute<shift> round trip (tests/tree.cpp:48-215)."""
    s = oracle.SU2()
    B = Qbasis.from_pairs(s, [(1, 1), (2, 1), (3, 1)])
    dom = B.combine(B)
    cod = B.combine(B)
    for q in dom.qs:
        if not cod.IS_PRESENT(q):
            continue
        for f1 in dom.trees[q]:
            for f2 in cod.trees[q]:
                for p in itertools.permutations(range(4)):
                    for shift in (-1, 0, 1):
                        acc = {}
                        for (g1, g2), c in treepair_permute(s, shift, f1, f2, list(p)).items():
                            for (h1, h2), c2 in treepair_permute(s, -shift, g1, g2, inverse_permutation(p)).items():
                                acc[(h1, h2)] = acc.get((h1, h2), 0.0) + c * c2
                        for k, c in acc.items():
                            assert abs(c - (1.0 if k == (f1, f2) else 0.0)) < 1e-12


def test_su2_6j_against_sympy():
    sympy = pytest.importorskip("sympy")
    from sympy.physics.wigner import wigner_6j
    rng = np.random.default_rng(0)
    n = 0
    tri = lambda x, y, z: (x + y + z) % 2 == 0 and abs(x - y) <= z <= x + y
    valid = [t for t in itertools.product(range(6), repeat=6)
             if tri(t[0], t[1], t[2]) and tri(t[0], t[4], t[5]) and tri(t[3], t[1], t[5]) and tri(t[3], t[4], t[2])]
    picks = [valid[i] for i in rng.choice(len(valid), size=250, replace=False)]
    picks += [tuple(int(x) for x in rng.integers(0, 7, size=6)) for _ in range(100)]
    for two in picks:
        try:
            ref = float(wigner_6j(*[sympy.Rational(t, 2) for t in two]))
        except ValueError:  # sympy rejects non-triangular arguments; the value is 0
            ref = 0.0
        assert abs(wigner6j_twice(*two) - ref) < 1e-14
        n += ref != 0.0
    assert n > 20


def test_permutation_decompose():
    for p in itertools.permutations(range(5)):
        a = list(range(5))
        for j in decompose_permutation(list(p)):
            a[j], a[j + 1] = a[j + 1], a[j]
        assert a == list(p)


def test_get_permutations_known_answers():
    # corner contraction C1T1 = C1.contract<{-1,1},{1,-2,-3,-4},1>(T1)  (CTM.cpp:1668)
    assert get_permutations([-1, 1], 0, [1, -2, -3, -4], 1, 1) == ([0, 1], -1, [0, 1, 2, 3], 0, [0, 1, 2, 3], 0)
    p1, s1, p2, s2, pres, sres = get_permutations([1, 2, -1, -2, 3], 2, [1, 2, 3, -3, -4], 3, 2)
    # A: Tensor<2,3> -> domain = open legs (2,3), codomain = contracted legs (0,1,4); shift 2-5+3 = 0
    assert (p1, s1, p2, s2, pres, sres) == ([2, 3, 0, 1, 4], 0, [0, 1, 2, 3, 4], 0, [0, 1, 2, 3], 0)


def test_tsvd_reconstruction_and_cutoff():
    rng = np.random.default_rng(1)
    s = oracle.U1()
    B = Qbasis.from_pairs(s, [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)])
    t = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    U, S, V, tw, ent = t.tsvd(10000, 0.0)
    rec = (U * S) * V
    for q in t.sectors:
        assert np.allclose(rec.block(q), t.block(q), atol=1e-12)
    U, S, V, tw, ent = t.tsvd(16, 1e-10)
    assert sum(b.shape[0] for b in S.blocks) == 16
    allsv = sorted(np.concatenate([np.linalg.svd(b, compute_uv=False) for b in t.blocks]), reverse=True)
    assert abs(tw - sum(x * x for x in allsv[16:])) < 1e-10 * tw
    kept = allsv[:16]
    assert abs(ent - sum(-x * x * np.log(x * x) for x in kept)) < 1e-10 * abs(ent)


def test_decompose_projector_identity():
    """P1 P2 is the identity on the kept space when nothing is truncated
    (decompose, PEPSContractions.cpp:16-43)."""
    rng = np.random.default_rng(2)
    s = oracle.U1()
    B = Qbasis.from_pairs(s, [(-1, 2), (0, 3), (1, 2)])
    t1 = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    t2 = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    P1, P2 = decompose(t1, t2, 10000)
    I = P1 * P2
    for q, b in zip(I.sectors, I.blocks):
        assert np.allclose(b, np.eye(b.shape[0]), atol=1e-9)


def test_permute_adj_is_the_adjoint_of_permute():
    """<permute(X), Y> == <X, permute_adj(Y)> on the stored entries
    (Tensor.cpp:258-333 is the transpose of permute_impl), for every
    permutation of a rank-4 tensor and shifts -1..1; U(1), fermionic U(1), SU(2)."""
    import itertools
    rng = np.random.default_rng(0)
    for sym in ("u1", "fu1", "su2"):
        s = oracle.make_symmetry(sym)
        legs = [Qbasis.from_pairs(s, random_pairs(rng, sym, 6 if sym != "su2" else 8), sort=True) for _ in range(4)]
        X = oracle.Tensor(s, legs[:2], legs[2:]).set_random(rng)
        for shift in (-1, 0, 1):
            for p in itertools.permutations(range(4)):
                Y = X.permute(shift, p)
                Yb = oracle.Tensor(s, Y.dom, Y.cod).set_random(rng)
                Xb = Yb.permute_adj(shift, p)
                assert Xb.sectors == X.sectors
                lhs, rhs = float(Y.data() @ Yb.data()), float(X.data() @ Xb.data())
                assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs)), (sym, shift, p)


def test_svd_backward_matches_finite_differences():
    """Reverse rule of the per-sector SVD (ADTensor.hpp:257-301) against
    central differences of <G_U, U> + <G_S, S> + <G_V, V^dag> with the sign
    gauge of fix_svd_signs, for square, tall and wide blocks."""
    import scipy.linalg as sla
    from oracle.tensor import fix_svd_signs, svd_backward_block
    rng = np.random.default_rng(0)
    for (m, n) in [(6, 6), (8, 5), (5, 8)]:
        A = rng.standard_normal((m, n))
        k = min(m, n)
        GU, GS, GV = rng.standard_normal((m, k)), np.diag(rng.standard_normal(k)), rng.standard_normal((k, n))

        def f(A):
            u, s, vt = sla.svd(A, full_matrices=False)
            u, vt = fix_svd_signs(u, vt)
            return (GU * u).sum() + (GS * np.diag(s)).sum() + (GV * vt).sum()

        u, s, vt = sla.svd(A, full_matrices=False)
        u, vt = fix_svd_signs(u, vt)
        dA = svd_backward_block(u, s, vt, GU, GS, GV)
        fd = np.zeros_like(A)
        for i in range(m):
            for j in range(n):
                E = np.zeros_like(A)
                E[i, j] = 1e-6
                fd[i, j] = (f(A + E) - f(A - E)) / 2e-6
        assert np.abs(fd - dA).max() <= 1e-7 * np.abs(fd).max()


def _diag_tensor(spectra):
    """Rank-(1,1) U(1) tensor whose sector q block is diag(spectra[q])."""
    s = oracle.U1()
    B = Qbasis.from_pairs(s, [(q, len(v)) for q, v in spectra])
    t = oracle.Tensor(s, [B], [B])
    for q, v in spectra:
        t.block(q)[:] = np.diag(v)
    return t


def test_cutoff_keeps_the_first_unsorted_value_when_eps_removes_all():
    """cutoff_matrices (Tensor.cpp:541-590): when eps removes every value the
    first entry of the unsorted list (the largest value of the first sector)
    is kept, not the global maximum; truncWeight sums the values beyond maxKeep."""
    t = _diag_tensor([(-1, [0.3, 0.1]), (0, [0.9, 0.2, 0.05]), (1, [0.4, 0.01])])
    U, S, V, tw, ent = t.tsvd(3, 10.0)
    assert S.sectors == [-1] and len(S.blocks) == 1
    assert S.blocks[0].shape == (1, 1) and abs(S.blocks[0][0, 0] - 0.3) < 1e-15
    assert abs(tw - (0.2 ** 2 + 0.1 ** 2 + 0.05 ** 2 + 0.01 ** 2)) < 1e-15
    assert abs(ent - (-0.09 * np.log(0.09))) < 1e-15


def test_cutoff_preserve_multiplets_cuts_at_the_last_relative_gap():
    """PRESERVE_MULTIPLETS (Tensor.cpp:568-582): scanning the kept values from
    the end, the cut moves to the last position whose relative gap
    2 (s_{i-1} - s_i) / (s_{i-1} + s_i) exceeds 0.1."""
    t = _diag_tensor([(-1, [1.0, 0.5]), (0, [0.9, 0.2, 0.19]), (1, [0.6, 0.195])])
    _, S, _, tw, ent = t.tsvd(6, 0.0, preserve_multiplets=True)
    kept = {q: sorted(np.diag(b).tolist(), reverse=True) for q, b in zip(S.sectors, S.blocks)}
    assert kept == {-1: [1.0, 0.5], 0: [0.9], 1: [0.6]}
    assert abs(tw - 0.19 ** 2) < 1e-15  # the weight counts only the values beyond maxKeep
    vals = [1.0, 0.9, 0.6, 0.5]
    assert abs(ent - sum(-v * v * np.log(v * v) for v in vals)) < 1e-14
    _, S2, _, _, _ = t.tsvd(6, 0.0, preserve_multiplets=False)
    assert sum(b.shape[0] for b in S2.blocks) == 6
