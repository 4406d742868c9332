"""Copies of device tensors as oracle tensors (test and baseline
infrastructure only): same leg bases, same sector order, same data."""
from __future__ import annotations

import numpy as np

from .basis import Qbasis
from .ctm import CTM, IPEPS
from .tensor import Tensor


def basis_from_native(sym, nb) -> Qbasis:
    qs, dims, conj, depth = nb.info()
    assert depth == 1, "only leg (depth 1) bases are converted"
    b = Qbasis(sym, 1)
    b.CONJ = bool(conj)
    for q, d in zip(qs, dims):
        b.push_back(int(q), int(d))
    b.IS_SORTED = list(qs) == sorted(qs)
    return b


def tensor_from_native(sym, nt) -> Tensor:
    r, c = nt.rank
    legs = [basis_from_native(sym, nt.leg(i)) for i in range(r + c)]
    ot = Tensor(sym, legs[:r], legs[r:])
    qs, rows, cols = nt.sectors()
    assert ot.sectors == list(qs), (ot.sectors, qs)
    flat = nt.data()
    o = 0
    for i, (m, n) in enumerate(zip(rows, cols)):
        assert ot.blocks[i].shape == (m, n)
        ot.blocks[i] = flat[o:o + m * n].reshape((m, n), order="F").copy()
        o += m * n
    return ot


def ctm_from_native(sym, nctm, chi) -> CTM:
    """Oracle CTM holding copies of a device CTM's site tensor and environment."""
    A = tensor_from_native(sym, nctm.get("A"))
    peps = IPEPS.__new__(IPEPS)
    peps.sym = sym
    peps.A = A
    peps.update_adag()
    oc = CTM(peps, chi)
    for k, t in nctm.env().items():
        setattr(oc, k, tensor_from_native(sym, t))
    return oc
