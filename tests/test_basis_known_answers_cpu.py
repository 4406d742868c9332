"""The reference's own Qbasis tests (tests/basis.cpp), restated for the oracle and
for the native library's leg bases:

* combine: for random bases B, C the full dimension (multiplicity times irrep
  dimension, summed) is multiplicative through B.C, B.C.B and B.C.B.C
  (tests/basis.cpp:31-79; random bases as Qbasis::setRandom, src/Core/Qbasis.cpp:93-103);
* push_back: pushing an irrep that is already present adds to its multiplicity,
  so a basis built from split pushes equals one built from the merged pushes
  (tests/basis.cpp:81-141).

The reference also runs these for the trivial symmetry U0, which this library
does not implement (no configuration uses it); fermionic Z2 stands in."""
import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from helpers import NAMES, random_pairs


def _native_full_dim(sym, basis):
    qs, ds, _, _ = basis.info()
    return sum(d * sym.degeneracy(q) for q, d in zip(qs, ds))


@pytest.mark.parametrize("symname", ["su2", "u1", "fz2"])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_combine_multiplies_full_dimensions(symname, seed):
    from xped_gb300 import Basis
    rng = np.random.default_rng(seed)
    s = oracle.make_symmetry(symname)
    pb, pc = random_pairs(rng, symname, 50, 5), random_pairs(rng, symname, 50, 5)
    B, C = Qbasis.from_pairs(s, pb), Qbasis.from_pairs(s, pc)
    nB, nC = Basis.from_pairs(NAMES[symname], pb), Basis.from_pairs(NAMES[symname], pc)
    b, c = B.fullDim(), C.fullDim()
    assert b == 50 and c == 50
    BC, nBC = B.combine(C), nB.combine(nC)
    assert BC.fullDim() == b * c == _native_full_dim(s, nBC)
    BCB, nBCB = BC.combine(B), nBC.combine(nB)
    assert BCB.fullDim() == b * c * b == _native_full_dim(s, nBCB)
    BCBC, nBCBC = BCB.combine(C), nBCB.combine(nC)
    assert BCBC.fullDim() == b * c * b * c == _native_full_dim(s, nBCBC)


# (vacuum, lowest_qs()[0], the irrep {5}) of each symmetry: SU(2) labels are 2j + 1, U(1) charges
IRREPS = {"su2": (1, 2, 5), "u1": (0, -1, 5), "fz2": (0, 1, 1)}


@pytest.mark.parametrize("symname", ["su2", "u1", "fz2"])
def test_push_back_merges_repeated_irreps(symname):
    from xped_gb300 import Basis
    vac, low, five = IRREPS[symname]
    s = oracle.make_symmetry(symname)
    if symname == "fz2":  # two irreps only: the third push goes to the odd one again
        merged = [(vac, 4), (low, 8 + 5)]
        split = [(vac, 1), (vac, 3), (low, 5), (low, 3), (five, 2), (five, 3)]
    else:
        merged = [(vac, 4), (low, 8), (five, 5)]
        split = [(vac, 1), (vac, 3), (low, 5), (low, 3), (five, 2), (five, 3)]
    B, C = Qbasis.from_pairs(s, merged, sort=False), Qbasis.from_pairs(s, split, sort=False)
    assert B == C
    nB = Basis.from_pairs(NAMES[symname], merged, sort=False)
    nC = Basis.from_pairs(NAMES[symname], split, sort=False)
    assert nB.info() == nC.info()
    assert nB.info()[:2] == (B.qs, B.dims)
    for i in range(len(B.qs)):
        assert nB.trees(i) == nC.trees(i)
