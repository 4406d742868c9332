"""GPU parity of the tensor operations against the CPU oracle, through the C-ABI.

Tolerances: permute/twist/adjoint are pure data movement with coefficients
+-1 (abelian) -> bit-exact; SU(2) coefficients are computed independently on
both sides -> 1e-13.  FP64 GEMM: 1e-12 relative to the block scale.  SVD:
gauge-normalised singular vectors and values to 1e-10 relative.
"""
import itertools

import numpy as np
import pytest

import oracle
from oracle.tensor import decompose as o_decompose
from helpers import assert_same, pair_basis, random_pairs, to_native

pytestmark = pytest.mark.gpu


def _pair_tensors(symname, pairsB, pairsC, seed=0):
    rng = np.random.default_rng(seed)
    s, oB, nB = pair_basis(symname, pairsB)
    _, oC, nC = pair_basis(symname, pairsC)
    ot = oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)
    nt = to_native(ot, [nB, nC], [nB, nC])
    return s, (oB, oC), (nB, nC), ot, nt


CASES = [
    ("u1", [(2, 2), (0, 1), (-1, 1), (-3, 1)], [(-2, 2), (1, 3)]),
    ("u1", [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)], [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)]),
    ("fu1", [(-1, 2), (0, 1), (1, 2), (2, 1)], [(0, 2), (1, 1), (-1, 1)]),
    ("fz2", [(0, 2), (1, 3)], [(1, 2), (0, 1)]),
    ("su2", [(1, 2), (2, 1), (3, 1)], [(1, 1), (2, 2)]),
]


@pytest.mark.parametrize("symname,pB,pC", CASES)
def test_permute_all(symname, pB, pC):
    s, ob, nb, ot, nt = _pair_tensors(symname, pB, pC)
    tol = 1e-13 if symname == "su2" else 0.0
    for p in itertools.permutations(range(4)):
        for shift in range(-2, 3):
            ref = ot.permute(shift, list(p))
            got = nt.permute(shift, list(p))
            assert_same(got, ref, rtol=tol, atol=tol)


# Larger degeneracies: the runs along output leg 0 are long enough (element-weighted 6-70) that the
# device takes its wide-row permute kernel (groups of 8-32 lanes) for these single-contribution plans,
# with rows both shorter than a group and longer than one pass of two elements per lane.
WIDE_CASES = [
    ("u1", [(-1, 3), (0, 20), (1, 5)], [(0, 9), (1, 35), (2, 2)]),
    ("fz2", [(0, 12), (1, 20)], [(0, 3), (1, 17)]),
]


@pytest.mark.parametrize("symname,pB,pC", WIDE_CASES)
def test_permute_wide_rows(symname, pB, pC):
    s, ob, nb, ot, nt = _pair_tensors(symname, pB, pC, seed=5)
    for p in itertools.permutations(range(4)):
        for shift in range(-2, 3):
            assert_same(nt.permute(shift, list(p)), ot.permute(shift, list(p)), rtol=0.0, atol=0.0)


def test_twist_then_permute():
    s, ob, nb, ot, nt = _pair_tensors("fu1", *CASES[2][1:])
    for mask in range(16):
        o2, n2 = ot, nt
        for l in range(4):
            if mask >> l & 1:
                o2, n2 = o2.twist(l), n2.twist(l)
        assert_same(n2.permute(1, [0, 2, 3, 1]), o2.permute(1, [0, 2, 3, 1]), 0, 0)
        assert_same(n2, o2, 0, 0)  # download materialises pending twists


def test_adjoint():
    for symname, pB, pC in CASES:
        s, ob, nb, ot, nt = _pair_tensors(symname, pB, pC)
        assert_same(nt.adjoint(), ot.adjoint(), 0, 0)


def test_matmul_and_adjoint_operands():
    rng = np.random.default_rng(3)
    s, oB, nB = pair_basis("u1", [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)])
    _, oC, nC = pair_basis("u1", [(-1, 3), (0, 5), (1, 2), (3, 1)])
    oT1 = oracle.Tensor(s, [oB, oB], [oC, oB]).set_random(rng)
    oT2 = oracle.Tensor(s, [oC, oB], [oB, oC]).set_random(rng)
    nT1 = to_native(oT1, [nB, nB], [nC, nB])
    nT2 = to_native(oT2, [nC, nB], [nB, nC])
    assert_same(nT1 * nT2, oT1 * oT2, 1e-12, 1e-12)
    # adjoint operands without materialising the transpose
    assert_same(nT1.matmul(nT1, adj_b=True), oT1 * oT1.adjoint(), 1e-12, 1e-12)
    assert_same(nT2.matmul(nT2, adj_a=True), oT2.adjoint() * oT2, 1e-12, 1e-12)


def test_tensor22_contract_permute_tsvd():
    """U(1) Tensor<2,2> op chain, legs q=-2..2 deg [2,4,6,4,2];
    T1*T2 -> permute<0>(0,2,1,3) -> tSVD(chi=16, eps=1e-10)."""
    pairs = [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)]
    for seed in range(3):
        rng = np.random.default_rng(seed)
        s, oB, nB = pair_basis("u1", pairs, sort=True)
        o1 = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
        o2 = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
        n1 = to_native(o1, [nB, nB], [nB, nB])
        n2 = to_native(o2, [nB, nB], [nB, nB])
        oprod = o1 * o2
        nprod = n1 * n2
        assert_same(nprod, oprod, 1e-12, 1e-12)
        operm = oprod.permute(0, [0, 2, 1, 3])
        nperm = nprod.permute(0, [0, 2, 1, 3])
        assert_same(nperm, operm, 1e-12, 1e-12)
        oU, oS, oV, otw, oent = operm.tsvd(16, 1e-10)
        nU, nS, nV, ntw, nent, keep = nperm.tSVD(16, 1e-10)
        assert_same(nS, oS, 1e-10, 1e-12)
        assert_same(nU, oU, 1e-9, 1e-9)
        assert_same(nV, oV, 1e-9, 1e-9)
        assert abs(ntw - otw) <= 1e-10 * max(1.0, otw)
        assert abs(nent - oent) <= 1e-10 * max(1.0, abs(oent))


def test_contract_labels():
    rng = np.random.default_rng(5)
    s, oB, nB = pair_basis("u1", [(-1, 1), (0, 2), (1, 1)], sort=True)
    _, oP, nP = pair_basis("u1", [(-1, 1), (1, 1)], sort=True)
    oA = oracle.Tensor(s, [oB, oB], [oB, oB, oP]).set_random(rng)
    nA = to_native(oA, [nB, nB], [nB, nB, nP])
    oAd = oA.adjoint().permute(0, [3, 4, 2, 0, 1])
    nAd = nA.adjoint().permute(0, [3, 4, 2, 0, 1])
    assert_same(nAd, oAd, 0, 0)
    for a1, a2, r in [([1, 2, -1, -2, 3], [1, 2, 3, -3, -4], 2), ([-1, 1, -2, -3, 2], [-4, 1, 2, -5, -6], 3),
                      ([-1, -2, 1, 2, 3], [-3, -4, 3, 1, 2], 2)]:
        assert_same(nA.contract(nAd, a1, a2, r), oA.contract(oAd, a1, a2, r), 1e-12, 1e-12)


def test_maxnorm_normalize():
    s, ob, nb, ot, nt = _pair_tensors(*CASES[1])
    assert nt.maxNorm() == ot.max_norm()
    assert_same(nt.normalize_max(), ot.normalize_max(), 0, 0)


def test_tsvd_truncation_edge_cases():
    rng = np.random.default_rng(11)
    s, oB, nB = pair_basis("u1", [(-1, 3), (0, 5), (1, 2)], sort=True)
    ot = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
    nt = to_native(ot, [nB, nB], [nB, nB])
    for keep, eps in [(1, 0.0), (7, 1e-10), (1000, 0.0), (1000, 1e-10), (40, 5.0), (3, 1e9)]:
        oU, oS, oV, otw, oent = ot.tsvd(keep, eps)
        nU, nS, nV, ntw, nent, _ = nt.tSVD(keep, eps)
        assert nS.sectors() == (oS.sectors, [b.shape[0] for b in oS.blocks], [b.shape[1] for b in oS.blocks])
        assert_same(nS, oS, 1e-10, 1e-12)
        assert_same(nU, oU, 1e-9, 1e-9)
        assert_same(nV, oV, 1e-9, 1e-9)


def test_tsvd_return_spec_matches_oracle():
    """RETURN_SPEC (Tensor.cpp:618-624): the per-sector kept singular values (SVspec) of the device tSVD
    against the oracle's cutoff_matrices with return_spec."""
    rng = np.random.default_rng(12)
    s, oB, nB = pair_basis("u1", [(-1, 3), (0, 5), (1, 2)], sort=True)
    ot = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
    nt = to_native(ot, [nB, nB], [nB, nB])
    for keep in (5, 17, 1000):
        *_, ospec = ot.tsvd(keep, 1e-10, return_spec=True)
        nspec = nt.tSVD(keep, 1e-10)[1].svspec()
        assert sorted(nspec) == sorted(ospec)
        for q, v in ospec.items():
            assert nspec[q].shape == v.shape
            assert np.abs(nspec[q] - v).max() <= 1e-10 * max(1.0, float(np.abs(v).max()))


def test_tsvd_preserve_multiplets_matches_oracle():
    """PRESERVE_MULTIPLETS (Tensor.cpp:568-582) on designed spectra: the kept
    list of 6 is cut back to 4 at the last relative gap above 0.1; truncWeight
    and entropy as the oracle gives them."""
    spectra = [(-1, [1.0, 0.5]), (0, [0.9, 0.2, 0.19]), (1, [0.6, 0.195])]
    s, oB, nB = pair_basis("u1", [(q, len(v)) for q, v in spectra], sort=True)
    ot = oracle.Tensor(s, [oB], [oB])
    for q, v in spectra:
        ot.block(q)[:] = np.diag(v)
    nt = to_native(ot, [nB], [nB])
    for keep, preserve in [(6, True), (6, False), (3, True), (100, True)]:
        oU, oS, oV, otw, oent = ot.tsvd(keep, 0.0, preserve_multiplets=preserve)
        nU, nS, nV, ntw, nent, _ = nt.tSVD(keep, 0.0, preserve)
        assert nS.sectors() == (oS.sectors, [b.shape[0] for b in oS.blocks], [b.shape[1] for b in oS.blocks])
        assert_same(nS, oS, 1e-14, 1e-15)
        assert abs(ntw - otw) <= 1e-14 and abs(nent - oent) <= 1e-14


def test_tqr():
    rng = np.random.default_rng(2)
    s, oB, nB = pair_basis("u1", [(-1, 3), (0, 5), (1, 2)], sort=True)
    _, oC, nC = pair_basis("u1", [(-1, 1), (0, 2), (1, 1)], sort=True)
    ot = oracle.Tensor(s, [oB, oB], [oC]).set_random(rng)  # tall blocks: middle = codomain
    nt = to_native(ot, [nB, nB], [nC])
    oQ, oR = ot.tqr()
    nQ, nR = nt.tQR()
    assert_same(nQ, oQ, 1e-11, 1e-11)
    assert_same(nR, oR, 1e-11, 1e-11)


def test_decompose_projectors():
    rng = np.random.default_rng(4)
    s, oB, nB = pair_basis("u1", [(-1, 2), (0, 3), (1, 2)], sort=True)
    o1 = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
    o2 = oracle.Tensor(s, [oB, oB], [oB, oB]).set_random(rng)
    n1 = to_native(o1, [nB, nB], [nB, nB])
    n2 = to_native(o2, [nB, nB], [nB, nB])
    oP1, oP2 = o_decompose(o1, o2, 12)
    from xped_gb300 import decompose
    nP1, nP2 = decompose(n1, n2, 12)
    assert_same(nP1, oP1, 1e-9, 1e-9)
    assert_same(nP2, oP2, 1e-9, 1e-9)


@pytest.mark.parametrize("symname,pB,pC", CASES)
def test_permute_adj_matches_oracle(symname, pB, pC):
    """permute_adj (Tensor.cpp:258-333) on cotangents shaped like permute's
    output, all permutations with shifts -1..1."""
    from oracle.convert import tensor_from_native
    from xped_gb300 import Tensor
    s, ob, nb, ot, nt = _pair_tensors(symname, pB, pC, seed=3)
    rng = np.random.default_rng(5)
    tol = 0 if symname != "su2" else 1e-13
    for shift in (-1, 0, 1):
        for p in itertools.permutations(range(4)):
            Y = nt.permute(shift, p)                      # forward output structure
            oY = tensor_from_native(s, Y)
            oYb = oracle.Tensor(s, oY.dom, oY.cod).set_random(rng)
            r, c = Y.rank
            nYb = Tensor.zeros([Y.leg(i) for i in range(r)], [Y.leg(i) for i in range(r, r + c)])
            nYb.set_data(oYb.data())
            assert_same(nYb.permute_adj(shift, p), oYb.permute_adj(shift, p), tol, tol)


@pytest.mark.parametrize("symname", ["u1", "fz2", "su2"])
def test_matmul_backward_matches_oracle(symname):
    """Reverse rule of operator* (ADTensor.hpp:741-752) with the operands'
    structures; includes sectors of `left` absent from the product."""
    rng = np.random.default_rng(9)
    pairs = {"u1": [(-1, 2), (0, 3), (1, 2)], "fz2": [(0, 2), (1, 3)], "su2": [(1, 2), (2, 1), (3, 1)]}[symname]
    pairs2 = {"u1": [(0, 2), (1, 1), (2, 1)], "fz2": [(0, 1), (1, 2)], "su2": [(1, 1), (2, 2)]}[symname]
    s, oB, nB = pair_basis(symname, pairs)
    _, oD, nD = pair_basis(symname, pairs2)
    oL = oracle.Tensor(s, [oB, oB], [oD]).set_random(rng)
    oR = oracle.Tensor(s, [oD], [oB]).set_random(rng)
    oC = oL * oR
    oCb = oracle.Tensor(s, oC.dom, oC.cod).set_random(rng)
    nL = to_native(oL, [nB, nB], [nD])
    nR = to_native(oR, [nD], [nB])
    nCb = to_native(oCb, [nB, nB], [nB])
    la, ra = nL.matmul_backward(nR, nCb)
    ola = oCb * oR.adjoint()
    ora = oL.adjoint() * oCb
    for nt, ref, like in ((la, ola, oL), (ra, ora, oR)):
        qs, rows, cols = nt.sectors()
        assert qs == like.sectors
        got = nt.blocks()
        for q in qs:
            want = ref.block(q) if ref.has(q) else np.zeros((rows[qs.index(q)], cols[qs.index(q)]))
            assert np.allclose(got[q], want, rtol=0, atol=1e-12 * max(1.0, np.abs(want).max()))


@pytest.mark.parametrize("symname", ["u1", "fz2", "su2"])
def test_svd_backward_matches_oracle(symname):
    """Reverse rule of the per-sector SVD (ADTensor.hpp:257-301) on the
    untruncated device tSVD factors, against the numpy restatement."""
    from oracle.convert import tensor_from_native
    from oracle.tensor import svd_backward_block
    from xped_gb300 import Tensor
    rng = np.random.default_rng(12)
    pairs = {"u1": [(-1, 2), (0, 3), (1, 2)], "fz2": [(0, 2), (1, 3)], "su2": [(1, 2), (2, 1), (3, 1)]}[symname]
    s, oB, nB = pair_basis(symname, pairs)
    oA = oracle.Tensor(s, [oB, oB], [oB]).set_random(rng)
    nA = to_native(oA, [nB, nB], [nB])
    U, S, V, *_ = nA.tSVD(10 ** 6, 0.0)

    def rand_like(t):
        r, c = t.rank
        z = Tensor.zeros([t.leg(i) for i in range(r)], [t.leg(i) for i in range(r, r + c)])
        z.set_data(rng.standard_normal(z.size))
        return z

    dU, dS, dV = rand_like(U), rand_like(S), rand_like(V)
    dA = nA.svd_backward(U, S, V, dU, dS, dV)
    oU, oS, oV = (tensor_from_native(s, t) for t in (U, S, V))
    odU, odS, odV = (tensor_from_native(s, t) for t in (dU, dS, dV))
    got = dA.blocks()
    for q in oA.sectors:
        ref = svd_backward_block(oU.block(q), np.diag(oS.block(q)), oV.block(q), odU.block(q), odS.block(q),
                                 odV.block(q))
        assert np.allclose(got[q], ref, rtol=0, atol=1e-10 * max(1.0, np.abs(ref).max())), q


@pytest.mark.parametrize("sizes", [[(520, 600), (40, 30)], [(700, 640), (1024, 1024)]])
def test_tsvd_wide_blocks_match_lapack(sizes):
    """Blocks at least 512 wide run on the grid-wide Jacobi kernel (the narrow ones of the same batch on
    the cluster kernel): singular values against LAPACK, full reconstruction, on graded spectra
    (sigma_i = 10^(-10 i / n)) that keep the Jacobi sweeps long."""
    from xped_gb300 import Basis, Tensor
    rng = np.random.default_rng(21)
    pairs_r = [(q, m) for q, (m, _n) in zip((-1, 1), sizes)]
    pairs_c = [(q, n) for q, (_m, n) in zip((-1, 1), sizes)]
    R, Cb = Basis.from_pairs("U1", pairs_r, sort=True), Basis.from_pairs("U1", pairs_c, sort=True)
    t = Tensor.zeros([R], [Cb])
    blocks, ref = [], []
    for m, n in sizes:
        k = min(m, n)
        u, _ = np.linalg.qr(rng.standard_normal((m, k)))
        v, _ = np.linalg.qr(rng.standard_normal((n, k)))
        s = 10.0 ** (-10.0 * np.arange(k) / k)
        blocks.append((u * s) @ v.T)
        ref.append(s)
    t.set_data(np.concatenate([b.ravel(order="F") for b in blocks]))
    U, S, V, _tw, _ent, keep = t.tSVD(1 << 30, 0.0)
    got = S.blocks()
    Ub, Vb = U.blocks(), V.blocks()
    for (q, _), blk, s in zip(pairs_r, blocks, ref):
        sv = np.diag(got[q])
        assert np.abs(sv - s).max() <= 1e-13 * s[0]
        rec = (Ub[q] * sv) @ Vb[q]
        assert np.abs(rec - blk).max() <= 1e-12 * np.abs(blk).max()


def test_tsvd_wide_block_matches_oracle_vectors():
    """A 560-wide U(1) sector (grid-wide Jacobi) next to narrower ones (cluster kernel): U, S, V^dag against
    the oracle's LAPACK tSVD with the shared sign rule, truncated to 200 values."""
    rng = np.random.default_rng(8)
    s, oB, nB = pair_basis("u1", [(-1, 24), (0, 40), (1, 24)], sort=True)
    _, oC, nC = pair_basis("u1", [(-1, 5), (0, 8), (1, 5)], sort=True)
    ot = oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)  # sectors 120 .. 560 wide
    nt = to_native(ot, [nB, nC], [nB, nC])
    assert max(min(b.shape) for b in ot.blocks) >= 512
    oU, oS, oV, otw, oent = ot.tsvd(200, 1e-10)
    nU, nS, nV, ntw, nent, _keep = nt.tSVD(200, 1e-10)
    assert_same(nS, oS, 1e-11, 1e-12)
    assert_same(nU, oU, 1e-8, 1e-9)
    assert_same(nV, oV, 1e-8, 1e-9)
    assert abs(ntw - otw) <= 1e-10 * max(1.0, otw)
