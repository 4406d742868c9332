"""CTMRG moves on the GPU against the oracle (1x1 cell, U(1) and fermionic Z2).

The SVD gauge is fixed identically on both sides (largest |u_i| positive), so
environments are compared entry by entry; tolerance 1e-8 relative after
several full steps (FP64 round-off accumulates through ~100 contractions and
four truncated SVDs per step)."""
import numpy as np
import pytest

from oracle.basis import Qbasis
from oracle.ctm import CTM as OCTM
from oracle.ctm import IPEPS
import oracle
from helpers import assert_same, pair_basis, to_native

pytestmark = pytest.mark.gpu


def _setup(symname, aux_pairs, phys_pairs, chi, seed):
    from xped_gb300 import CTM
    s, oaux, naux = pair_basis(symname, aux_pairs, sort=True)
    _, ophys, nphys = pair_basis(symname, phys_pairs, sort=True)
    rng = np.random.default_rng(seed)
    peps = IPEPS(s, oaux, ophys).set_random(rng)
    nA = to_native(peps.A, [naux, naux], [naux, naux, nphys])
    return OCTM(peps, chi).init(), CTM(nA, chi).init()


def _compare(oc, nc, rtol):
    env = oc.env()
    for name, t in nc.env().items():
        assert_same(t, env[name], rtol, rtol)


def test_ctm_init_u1():
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 8, 0)
    _compare(oc, nc, 1e-12)
    assert_same(nc.get("Adag"), oc.peps.Adag, 0, 0)


@pytest.mark.parametrize("seed", [0, 1])
def test_ctm_steps_u1_small(seed):
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 12, seed)
    for _ in range(3):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-8)


def test_ctm_config2_step():
    """BASELINE config 2: U(1), phys dim 2, D=4 (q -1..1 deg [1,2,1]), chi=32."""
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    for _ in range(2):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-8)


def test_ctm_fermionic_z2():
    oc, nc = _setup("fz2", [(0, 2), (1, 2)], [(0, 1), (1, 1)], 10, 3)
    _compare(oc, nc, 1e-12)
    for _ in range(2):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-8)
