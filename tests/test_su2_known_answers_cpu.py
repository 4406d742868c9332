"""The oracle's SU(2) algebra pinned by the reference's own known answers
(tests/tensor.cpp:230-385, tests/tensor_tests.hpp:1-48,305-333):
  * plainTensor (src/Core/Tensor.cpp:1133-1310, Clebsch-Gordan tensors of
    src/Symmetry/SU2.cpp:42-89 with dual legs bent by the 1j tensor,
    src/Core/FusionTree.cpp:155-285) preserves the squared norm;
  * permute<shift, p> of an SU(2) Tensor<2,2> equals the dense shuffle of its
    plainTensor for every permutation and shift -2..2;
  * reduced spin operators expand to the spin matrices, S.S = S(S+1), the
    K=1 and K=2 couplings and S1.S2 in every total-spin sector, 2S = 1..10."""
import itertools

import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from su2_known import OracleBackend, check_outer_product, check_spin_known_answers

S = oracle.make_symmetry("su2")


def _rank4(seed):
    rng = np.random.default_rng(seed)
    B = Qbasis.from_pairs(S, [(1, 1), (2, 2), (3, 1)])
    C = Qbasis.from_pairs(S, [(2, 1), (1, 1), (4, 1)])
    return oracle.Tensor(S, [B, C], [B, C]).set_random(rng)


def test_plain_tensor_keeps_the_squared_norm():
    t = _rank4(0)
    P = t.plain_tensor()
    assert abs(float(np.sum(P * P)) - t.squared_norm()) < 1e-10 * t.squared_norm()


@pytest.mark.parametrize("shift", [-2, -1, 0, 1, 2])
def test_su2_permute_equals_dense_shuffle(shift):
    t = _rank4(1)
    P = t.plain_tensor()
    for p in itertools.permutations(range(4)):
        got = t.permute(shift, list(p)).plain_tensor()
        assert np.abs(got - np.transpose(P, p)).max() < 1e-12, (shift, p)


def test_u1_fermionic_plain_is_unchanged_by_bending():
    """Abelian symmetries: the 1j tensor is 1, so plainTensor is the sub-block placement."""
    s = oracle.make_symmetry("u1")
    rng = np.random.default_rng(2)
    B = Qbasis.from_pairs(s, [(-1, 1), (0, 2), (1, 1)])
    t = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    P = t.plain_tensor()
    for p in itertools.permutations(range(4)):
        for shift in (-1, 1):
            assert np.abs(t.permute(shift, list(p)).plain_tensor() - np.transpose(P, p)).max() < 1e-13


@pytest.mark.parametrize("two_s", list(range(1, 11)))
def test_spin_operator_known_answers(two_s):
    assert check_spin_known_answers(OracleBackend(), two_s) < 1e-10


def test_spin_outer_products():
    worst = 0.0
    for a in range(1, 11):
        for b in range(1, 11):
            worst = max(worst, check_outer_product(OracleBackend(), a, b))
    assert worst < 1e-10
