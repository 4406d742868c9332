"""The reference's SU(2) known answers on the device (tests/tensor.cpp:230-385,
tests/tensor_tests.hpp:1-48): the same operator chains as
test_su2_known_answers_cpu.py, every permute and product run by this library's
kernels through the C-ABI, the results expanded to dense tensors on the host
(plainTensor with SU(2) Clebsch-Gordan tensors) and compared with the spin
matrices; and the device permute of a random SU(2) Tensor<2,2> against the dense
shuffle of its plainTensor for every permutation and shift -2..2."""
import itertools

import numpy as np
import pytest

import oracle
from oracle.convert import tensor_from_native
from su2_known import SYM, DeviceBackend, OracleBackend, check_outer_product, check_spin_known_answers

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _device():
    from xped_gb300 import ensure_device
    ensure_device(0)


@pytest.mark.parametrize("two_s", list(range(1, 11)))
def test_spin_operator_known_answers_on_device(two_s):
    assert check_spin_known_answers(DeviceBackend(), two_s) < 1e-10


def test_spin_outer_products_on_device():
    worst = 0.0
    for a in range(1, 11):
        for b in (1, 2, 5, 10):
            worst = max(worst, check_outer_product(DeviceBackend(), a, b))
    assert worst < 1e-10


@pytest.mark.parametrize("shift", [-2, -1, 0, 1, 2])
def test_su2_device_permute_equals_dense_shuffle(shift):
    from xped_gb300 import Basis, Tensor
    pb, pc = [(1, 1), (2, 2), (3, 1)], [(2, 1), (1, 1), (4, 1)]
    B, C = Basis.from_pairs("SU2", pb), Basis.from_pairs("SU2", pc)
    t = Tensor.zeros([B, C], [B, C])
    t.set_data(np.random.default_rng(5).standard_normal(t.size))
    P = tensor_from_native(SYM, t).plain_tensor()
    for p in itertools.permutations(range(4)):
        got = tensor_from_native(SYM, t.permute(shift, list(p))).plain_tensor()
        assert np.abs(got - np.transpose(P, p)).max() < 1e-12, (shift, p)


def test_device_chain_matches_oracle_chain():
    """The K=2 coupled product of spin 3/2 on the device equals the oracle's, entry by entry."""
    from su2_known import coupled_product, spin_operator
    dev, orc = DeviceBackend(), OracleBackend()
    d = coupled_product(dev, spin_operator(dev, 3)[0], 5)
    o = coupled_product(orc, spin_operator(orc, 3)[0], 5)
    assert np.abs(d.data() - o.data()).max() < 1e-13
