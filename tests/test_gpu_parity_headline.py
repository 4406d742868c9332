"""CTMRG parity at the benchmark's own configurations and at the FP64 contract
tolerance of 1e-10 relative.

The U(1) iPEPS of the headline benchmark (physical q -1/+1, virtual D=6 with
q -1,0,1 and degeneracies [2,2,2], chi=128, N(0,1) site tensor from seed 1234,
FROM_A start) runs two plain FP64 steps (grow_all: left, right, top and bottom
moves, src/PEPS/CTM.cpp:385-420,924-1183) on the device and in the oracle;
every environment tensor (C1..C4, T1..T4) is compared entry by entry.  The
same check runs for the fermionic Z2 iPEPS of the full chosen-form
configuration (D=6 with q 0,1 and degeneracies [3,3]) at chi=24, a size the
oracle finishes in seconds.  The environments are normalised by their largest
entry (src/PEPS/CTM.cpp:1372), so the tolerance is relative to the largest
entry of each tensor."""
import numpy as np
import pytest

from oracle.ctm import CTM as OCTM
from oracle.ctm import IPEPS
from helpers import assert_same, pair_basis, to_native

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _setup(symname, aux_pairs, phys_pairs, chi, seed):
    from xped_gb300 import CTM
    s, oaux, naux = pair_basis(symname, aux_pairs, sort=True)
    _, ophys, nphys = pair_basis(symname, phys_pairs, sort=True)
    peps = IPEPS(s, oaux, ophys).set_random(np.random.default_rng(seed))
    nA = to_native(peps.A, [naux, naux], [naux, naux, nphys])
    return OCTM(peps, chi).init(), CTM(nA, chi).init()


def _max_err(oc, nc):
    env = oc.env()
    worst = 0.0
    for name, t in nc.env().items():
        worst = max(worst, assert_same(t, env[name], RTOL, RTOL))
    return worst


def _env_err(oc, nc):
    env = oc.env()
    return max(float(np.abs(t.data() - env[n].data()).max()) for n, t in nc.env().items())


def test_headline_u1_D6_chi128_two_plain_steps():
    """The FROM_A start of this configuration meets exactly degenerate singular values in its first
    decompositions (relative gaps 0 and 4e-16 among the kept values): there LAPACK and the device
    Jacobi SVD may pick different orthonormal bases of a degenerate pair, a rotation of the new chi
    leg that changes no observable.  So after the first step the gauge-invariant reduced density
    matrices and energies are compared (1e-12), and the environments entry by entry after the
    second step, whose moves re-project every chi leg through non-degenerate decompositions
    (measured: 3.4e-10 after step 1, 1.5e-11 after step 2)."""
    from oracle.ctm import bond_expectation as obond
    from oracle.ctm import heisenberg_u1
    import oracle
    from xped_gb300 import bond_expectation
    from xped_gb300.observables import heisenberg_bond
    oc, nc = _setup("u1", [(-1, 2), (0, 2), (1, 2)], [(-1, 1), (1, 1)], 128, 1234)
    assert _env_err(oc, nc) == 0.0
    H = heisenberg_bond(nc.get("A").leg(4))
    oH = heisenberg_u1(oracle.make_symmetry("u1"), oc.peps.A.cod[2])
    errs = []
    for step in range(2):
        oc.grow_all()
        nc.grow_all()
        errs.append(_env_err(oc, nc))
        for orho, nrho in ((oc.rdm_h(), nc.rdm_h()), (oc.rdm_v(), nc.rdm_v())):
            assert_same(nrho, orho, 1e-12, 1e-12)
            assert abs(bond_expectation(nrho, H) - obond(orho, oH)) < 1e-12
    print("U(1) D=6 chi=128: largest environment difference after step 1 / step 2:", errs)
    _max_err(oc, nc)  # every tensor within 1e-10 after the second step


def test_fermionic_z2_D6_chi24_plain_steps():
    oc, nc = _setup("fz2", [(0, 3), (1, 3)], [(0, 1), (1, 1)], 24, 1234)
    errs = [_max_err(oc, nc)]
    for _ in range(3):
        oc.grow_all()
        nc.grow_all()
        errs.append(_max_err(oc, nc))
    print("fermionic Z2 D=6 chi=24: largest environment difference after init / steps 1-3:", errs)
