"""CPU checks of the simple-update restatement (oracle/simple_update.py): the
unit-cell pattern arithmetic of the reference (Pattern.cpp) and the invariants
of a bond update (normalised weights, truncation to D, exp of a block-diagonal
operator)."""
import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from oracle.ctm import IPEPS, heisenberg_u1
from oracle.simple_update import Pattern, SimpleUpdate, gate


def test_pattern_wraps_and_orders_sites_like_the_reference():
    # Pattern::index(x, y) = x + y Lx after wrapping; coords(i) = (i % Lx, i / Lx)
    p = Pattern([[0, 1], [1, 0]])
    assert (p.Lx, p.Ly, p.n) == (2, 2, 2)
    assert [p.coords(i) for i in range(2)] == [(0, 0), (1, 0)]
    assert p.label(-1, 0) == p.label(1, 0) == 1
    assert p.label(0, -1) == p.label(0, 1) == 1
    assert p.label(2, 2) == p.label(0, 0) == 0
    q = Pattern([[0, 1, 2]])  # Lx = 1, Ly = 3
    assert [q.coords(i) for i in range(3)] == [(0, 0), (0, 1), (0, 2)]


def test_gate_is_the_exponential_of_every_block():
    s = oracle.make_symmetry("u1")
    phys = Qbasis.from_pairs(s, [(-1, 1), (1, 1)])
    H = heisenberg_u1(s, phys)
    U = gate(H, 0.3)
    for b, u in zip(H.blocks, U.blocks):
        w, v = np.linalg.eigh(b)
        assert np.allclose(u, (v * np.exp(-0.3 * w)) @ v.T, atol=1e-14)


@pytest.mark.parametrize("symname,aux_p,phys_p", [
    ("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)]),
    ("fz2", [(0, 2), (1, 2)], [(0, 1), (1, 1)]),
])
def test_bond_update_normalises_and_truncates(symname, aux_p, phys_p):
    s = oracle.make_symmetry(symname)
    aux, phys = Qbasis.from_pairs(s, aux_p), Qbasis.from_pairs(s, phys_p)
    rng = np.random.default_rng(2)
    Gs = [IPEPS(s, aux, phys).set_random(rng).A for _ in range(2)]
    if symname == "u1":
        U = gate(heisenberg_u1(s, phys), 0.05)
    else:
        U = Gs[0].identity(s, [phys, phys], [phys, phys])
    su = SimpleUpdate([[0, 1], [1, 0]], Gs, 3).step(U, U)
    for w in su.wh + su.wv:
        d = np.concatenate([np.diag(b) for b in w.blocks])
        assert 0 < d.size <= 3
        assert abs(d.max() - 1.0) < 1e-15 and d.min() > 0.0
    # the bond legs of the site tensors carry the truncated weight bases
    for i in range(2):
        g = su.G[i]
        assert g.cod[0].fullDim() == su.wh[i].dom[0].fullDim()
        assert g.dom[1].fullDim() == su.wv[i].dom[0].fullDim()
