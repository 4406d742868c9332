"""Shared helpers: build matching oracle / native bases and tensors from the
same seeded inputs."""
from __future__ import annotations

import numpy as np

import oracle
from oracle.basis import Qbasis

NAMES = {"u1": "U1", "fu1": "fU1", "z2": "Z2", "fz2": "fZ2", "su2": "SU2"}


def pair_basis(symname, pairs, sort=False):
    from xped_gb300 import Basis
    s = oracle.make_symmetry(symname)
    return s, Qbasis.from_pairs(s, pairs, sort=sort), Basis.from_pairs(NAMES[symname], pairs, sort=sort)


def random_pairs(rng, symname, full_dim, max_sector=3):
    """Random leg basis like Qbasis::setRandom (Qbasis.cpp:93-103), seeded."""
    s = oracle.make_symmetry(symname)
    pairs, tot = [], 0
    seen = {}
    while tot < full_dim:
        if symname in ("u1", "fu1"):
            q = int(rng.integers(-3, 4))
        elif symname in ("z2", "fz2"):
            q = int(rng.integers(0, 2))
        else:
            q = int(rng.integers(1, 5))
        d = int(rng.integers(1, max_sector + 1))
        if tot + s.degeneracy(q) * d <= full_dim:
            pairs.append((q, d))
            tot += s.degeneracy(q) * d
            seen[q] = True
    return pairs


def to_native(ot, dom, cod):
    """Upload an oracle tensor into a native tensor with the same bases."""
    from xped_gb300 import Tensor
    nt = Tensor.zeros(dom, cod)
    qs = nt.sectors()[0]
    assert qs == ot.sectors, (qs, ot.sectors)
    nt.set_data(ot.data())
    return nt


def assert_same(nt, ot, rtol=1e-12, atol=1e-12):
    qs, rs, cs = nt.sectors()
    assert qs == ot.sectors, (qs, ot.sectors)
    got = nt.data()
    ref = ot.data()
    assert got.shape == ref.shape
    scale = max(1.0, float(np.abs(ref).max()) if ref.size else 1.0)
    err = float(np.abs(got - ref).max()) if ref.size else 0.0
    assert err <= atol + rtol * scale, f"max abs err {err:.3e} (scale {scale:.3e})"
    return err
