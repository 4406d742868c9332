"""Simple-update imaginary-time step (TimePropagator::t_step_h / t_step_v) on
the GPU against the CPU restatement, on the checkerboard unit cell
[[0, 1], [1, 0]] (the reference requires neighbouring sites to differ), from
the same site tensors and gates.  Every tSVD on both sides uses the same sign
rule, so site tensors and bond weights are compared element by element."""
import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from oracle.ctm import IPEPS, heisenberg_u1
from oracle.simple_update import SimpleUpdate as OSU
from oracle.simple_update import gate
from oracle.tensor import Tensor as OTensor

from helpers import assert_same, to_native

pytestmark = pytest.mark.gpu

CHECKERBOARD = [[0, 1], [1, 0]]


def _density(sym, phys):
    """V n1 n2 for parity charges 0 (empty) / 1 (occupied), built in the oracle."""
    H = OTensor(sym, [phys, phys], [phys, phys])
    for i, q in enumerate(H.sectors):
        rows = [tuple(t.qu) for t in H.cdom.trees[q]]
        cols = [tuple(t.qu) for t in H.ccod.trees[q]]
        H.blocks[i] = np.array([[1.0 if (a == b and a == (1, 1)) else 0.0 for b in cols] for a in rows])
    return H


def _setup(symname, aux_p, phys_p, seed, tau=0.05):
    from xped_gb300 import Basis
    names = {"u1": "U1", "fz2": "fZ2"}
    s = oracle.make_symmetry(symname)
    oaux, ophys = Qbasis.from_pairs(s, aux_p), Qbasis.from_pairs(s, phys_p)
    naux, nphys = Basis.from_pairs(names[symname], aux_p), Basis.from_pairs(names[symname], phys_p)
    rng = np.random.default_rng(seed)
    oG = [IPEPS(s, oaux, ophys).set_random(rng).A for _ in range(2)]
    nG = [to_native(g, [naux, naux], [naux, naux, nphys]) for g in oG]
    H = heisenberg_u1(s, ophys) if symname == "u1" else _density(s, ophys)
    U = gate(H, tau)
    nU = to_native(U, [nphys, nphys], [nphys, nphys])
    return oG, nG, U, nU


def _compare(nsu, osu, rtol):
    for i in range(2):
        assert_same(nsu.get("wh", i), osu.wh[i], rtol, 1e-12)
        assert_same(nsu.get("wv", i), osu.wv[i], rtol, 1e-12)
        assert_same(nsu.get("G", i), osu.G[i], rtol, 1e-12)


@pytest.mark.parametrize("symname,aux_p,phys_p,D", [
    ("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 3),
    ("u1", [(-1, 2), (0, 2), (1, 2)], [(-1, 1), (1, 1)], 6),
    ("fz2", [(0, 2), (1, 2)], [(0, 1), (1, 1)], 3),
])
def test_simple_update_matches_oracle(symname, aux_p, phys_p, D):
    from xped_gb300 import SimpleUpdate, ensure_device
    ensure_device(0)
    oG, nG, oU, nU = _setup(symname, aux_p, phys_p, seed=11)
    osu, nsu = OSU(CHECKERBOARD, oG, D), SimpleUpdate(CHECKERBOARD, nG, D)
    osu.step_h(0, 0, oU)
    nsu.step_h(0, 0, nU)
    _compare(nsu, osu, 1e-9)
    osu.step_v(1, 0, oU)
    nsu.step_v(1, 0, nU)
    _compare(nsu, osu, 1e-9)
    for _ in range(2):
        osu.step(oU, oU)
        nsu.step(nU, nU)
    _compare(nsu, osu, 1e-8)
    for i in range(2):
        assert_same(nsu.get("A", i), osu.site_tensor(i), 1e-8, 1e-12)


def test_weights_are_normalised_and_truncated():
    """Bond weights after a step: largest entry 1 (weight * (1 / maxNorm)),
    at most D values, all positive."""
    from xped_gb300 import SimpleUpdate, ensure_device
    ensure_device(0)
    _oG, nG, _oU, nU = _setup("u1", [(-1, 2), (0, 2), (1, 2)], [(-1, 1), (1, 1)], seed=3)
    nsu = SimpleUpdate(CHECKERBOARD, nG, 4).step(nU, nU)
    for i in range(2):
        for name in ("wh", "wv"):
            d = np.concatenate([np.diag(b) for b in nsu.get(name, i).blocks().values()])
            assert d.size <= 4
            assert abs(d.max() - 1.0) < 1e-15
            assert d.min() > 0.0


def test_pattern_with_equal_neighbours_is_rejected():
    from xped_gb300 import SimpleUpdate, XgbError, ensure_device
    ensure_device(0)
    _oG, nG, _oU, _nU = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], seed=5)
    with pytest.raises(XgbError):
        SimpleUpdate([[0]], nG[:1], 3)
