"""SU(2) known answers of the reference's own tests, restated: reduced spin-S
operators built as SU(2) tensors must, through permute (with turns) and
operator*, expand (plainTensor) to the spin matrices, S^2 = S(S+1), and the
rank-1 / rank-2 couplings of two spin operators (tests/tensor.cpp:230-385).
The chains are written once against a small backend interface so that the
same steps run on the oracle (CPU) and on the device tensors."""
from __future__ import annotations

import numpy as np

import oracle
from oracle.basis import Qbasis
from oracle.convert import tensor_from_native

SYM = oracle.make_symmetry("su2")


class OracleBackend:
    def basis(self, pairs):
        return Qbasis.from_pairs(SYM, pairs)

    def constant(self, dom, cod, value):
        t = oracle.Tensor(SYM, dom, cod)
        t.blocks = [np.full(b.shape, float(value)) for b in t.blocks]
        return t

    def plain(self, t):
        return t.plain_tensor()

    def data(self, t):
        return t.data()


class DeviceBackend:
    def basis(self, pairs):
        from xped_gb300 import Basis
        return Basis.from_pairs("SU2", pairs)

    def constant(self, dom, cod, value):
        from xped_gb300 import Tensor
        t = Tensor.zeros(dom, cod)
        t.set_data(np.full(t.size, float(value)))
        return t

    def plain(self, t):
        return tensor_from_native(SYM, t).plain_tensor()

    def data(self, t):
        return t.data()


def spin_matrices(two_s):
    """The spherical components (-S+/sqrt2, Sz, S-/sqrt2) of spin S = two_s / 2,
    basis ordered m = S, S-1, ..., -S (tests/tensor.cpp:251-277)."""
    S = 0.5 * two_s
    n = two_s + 1
    p = [np.zeros((n, n)) for _ in range(3)]
    for i in range(1, n):
        m = S - i
        p[0][i - 1, i] = np.sqrt(S * (S + 1) - m * (m + 1))
    p[0] *= -np.sqrt(0.5)
    for i in range(n):
        p[1][i, i] = S - i
    for i in range(n - 1):
        m = S - i
        p[2][i + 1, i] = np.sqrt(S * (S + 1) - m * (m - 1))
    p[2] *= np.sqrt(0.5)
    return p


def spin_operator(be, two_s):
    """Reduced spin-S operator: Tensor<2,1>({B, C}, {B}) with B = irrep 2S+1,
    C = irrep 3 (spin 1), every entry sqrt(S(S+1))."""
    S = 0.5 * two_s
    B = be.basis([(two_s + 1, 1)])
    C = be.basis([(3, 1)])
    return be.constant([B, C], [B], np.sqrt(S * (S + 1.0))), B, C


def coupled_product(be, s1, K2p1):
    """(s1^dag.permute<-1,0,1,2>() * couple.permute<+1,0,2,1>()).permute<0,0,3,1,2>() * s1
    with couple = Tensor<2,1>({C, K}, {C}) all ones (tests/tensor.cpp:301-302)."""
    C = be.basis([(3, 1)])
    K = be.basis([(K2p1, 1)])
    couple = be.constant([C, K], [C], 1.0)
    x = s1.adjoint().permute(-1, [0, 1, 2]) * couple.permute(+1, [0, 2, 1])
    return x.permute(0, [0, 3, 1, 2]) * s1


def check_spin_known_answers(be, two_s, tol=1e-12):
    """Returns the largest deviation from the known answers for spin two_s / 2."""
    S = 0.5 * two_s
    n = two_s + 1
    pv = spin_matrices(two_s)
    s1, _, _ = spin_operator(be, two_s)
    worst = 0.0
    # the reduced operator expands to the spin matrices (tests/tensor.cpp:283-297)
    tp = be.plain(s1.adjoint())
    assert tp.shape == (n, n, 3)
    for k in range(3):
        worst = max(worst, float(np.linalg.norm(tp[:, :, k] - pv[k])))
    # K = 0: S.S = S(S+1) on the diagonal (tests/tensor.cpp:300-317)
    c1 = be.plain(coupled_product(be, s1, 1))
    assert c1.shape == (n, 1, n)
    worst = max(worst, float(np.linalg.norm(c1[:, 0, :] - S * (S + 1.0) * np.eye(n))))
    # K = 1: (S x S)^1 = sqrt(1/2) S (tests/tensor.cpp:319-335)
    c3 = be.plain(coupled_product(be, s1, 3).adjoint())
    assert c3.shape == (n, n, 3)
    for k in range(3):
        worst = max(worst, float(np.linalg.norm(c3[:, :, k] - np.sqrt(0.5) * pv[k])))
    # K = 2: the quadrupole components (tests/tensor.cpp:336-357)
    c5 = be.plain(coupled_product(be, s1, 5).adjoint())
    assert c5.shape == (n, n, 5)
    q = [-np.sqrt(0.6) * (pv[0] @ pv[0]),
         -np.sqrt(0.3) * (pv[0] @ pv[1] + pv[1] @ pv[0]),
         -np.sqrt(0.1) * (pv[0] @ pv[2] + pv[2] @ pv[0] + 2 * pv[1] @ pv[1]),
         -np.sqrt(0.3) * (pv[2] @ pv[1] + pv[1] @ pv[2]),
         -np.sqrt(0.6) * (pv[2] @ pv[2])]
    for k in range(5):
        worst = max(worst, float(np.linalg.norm(c5[:, :, k] - q[k])))
    return worst


def check_outer_product(be, two_s1, two_s2):
    """S1.S2 coupled to total spin: every sector of the outer product is 1 x 1 and
    equals (Stot(Stot+1) - S1(S1+1) - S2(S2+1)) / 2 (tests/tensor.cpp:360-381).
    Returns the largest deviation."""
    S1, S2 = 0.5 * two_s1, 0.5 * two_s2
    s1, _, _ = spin_operator(be, two_s1)
    s2, _, _ = spin_operator(be, two_s2)
    C = be.basis([(3, 1)])
    one = be.basis([(1, 1)])
    couple = be.constant([C, one], [C], 1.0)
    x = (s1.adjoint().permute(-1, [0, 1, 2]) * couple.permute(+1, [0, 2, 1])).permute(-1, [0, 1, 3, 2])
    out = (x * s2.permute(+1, [1, 2, 0])).permute(0, [0, 4, 2, 1, 3])
    worst = 0.0
    qs, rows, cols = sectors_of(out)
    flat = be.data(out)
    o = 0
    for q, r, c in zip(qs, rows, cols):
        assert r * c == 1, (q, r, c)
        Stot = 0.5 * (q - 1)
        want = 0.5 * (Stot * (Stot + 1) - S1 * (S1 + 1.0) - S2 * (S2 + 1.0))
        worst = max(worst, abs(float(flat[o]) - want))
        o += r * c
    assert len(qs) == min(two_s1, two_s2) + 1
    return worst


def sectors_of(t):
    if hasattr(t, "blocks") and isinstance(t.blocks, list):
        return list(t.sectors), [b.shape[0] for b in t.blocks], [b.shape[1] for b in t.blocks]
    return t.sectors()
