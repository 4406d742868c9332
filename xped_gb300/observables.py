"""Two-site operators for bond energies of the CTM environments.

``heisenberg_bond`` is the spin-1/2 Heisenberg coupling
J (Sz Sz + (S+ S- + S- S+) / 2) as a U(1) Tensor<2,2>({phys, phys}, {phys, phys})
with phys charges 2 Sz = -1, +1 (degeneracy 1 each), built block by block in
the coupled sectors' fusion-tree row order; ``density_bond`` is V n_1 n_2 for
parity charges 0/1.  ``energy`` is the bond energy per
site of a 1x1 cell: the horizontal plus the vertical bond expectation
(avg, src/PEPS/LinearAlgebra.cpp:58-80)."""
from __future__ import annotations

import numpy as np

from .tensor import Basis, CTM, Tensor, bond_expectation


def _rows(coupled: Basis, q: int):
    qs = coupled.qs
    out = []
    for qu, _qi, _qc, dims, _dual in coupled.trees(qs.index(q)):
        if any(d != 1 for d in dims):
            raise ValueError("heisenberg_bond needs a spin-1/2 leg with degeneracy 1 per charge")
        out.append(qu)
    return out


def heisenberg_bond(phys: Basis, J: float = 1.0) -> Tensor:
    if sorted(phys.qs) != [-1, 1]:
        raise ValueError("heisenberg_bond needs physical charges -1, +1 (2 Sz)")
    sz = {-1: -0.5, 1: 0.5}
    H = Tensor.zeros([phys, phys], [phys, phys])
    cd, cc = H.coupled(False), H.coupled(True)
    blocks = {}
    for q in H.sectors()[0]:
        rows, cols = _rows(cd, q), _rows(cc, q)
        b = np.zeros((len(rows), len(cols)))
        for r, (a1, a2) in enumerate(rows):
            for c, (b1, b2) in enumerate(cols):
                v = sz[a1] * sz[a2] if (a1, a2) == (b1, b2) else 0.0
                if a1 == b2 and a2 == b1 and a1 != a2:
                    v += 0.5
                b[r, c] = J * v
        blocks[q] = b
    H.set_blocks(blocks)
    return H


def density_bond(phys: Basis, V: float = 1.0) -> Tensor:
    """V n_1 n_2 for a spinless-fermion (or hard-core) site with parity charges
    0 (empty) and 1 (occupied), degeneracy 1 each: diagonal, parity even."""
    if sorted(phys.qs) != [0, 1]:
        raise ValueError("density_bond needs physical charges 0, 1")
    H = Tensor.zeros([phys, phys], [phys, phys])
    cd, cc = H.coupled(False), H.coupled(True)
    blocks = {}
    for q in H.sectors()[0]:
        rows, cols = _rows(cd, q), _rows(cc, q)
        b = np.zeros((len(rows), len(cols)))
        for r, a in enumerate(rows):
            for c, bb in enumerate(cols):
                if a == bb and a == (1, 1):
                    b[r, c] = V
        blocks[q] = b
    H.set_blocks(blocks)
    return H


def energy(ctm: CTM, H: Tensor) -> float:
    return bond_expectation(ctm.rdm_h(), H) + bond_expectation(ctm.rdm_v(), H)
