"""CPU-side checks of the native library: it loads, exports every symbol the
headers declare, and its host metadata (bases, fusion trees, sector order,
permute and GEMM plans) matches the oracle bit for bit.  The permute plans
are executed here by a numpy emulation of the kernel's index arithmetic."""
import itertools
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle.tensor import get_permutations
from helpers import pair_basis

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    import ctypes
    from xped_gb300._lib import LIB_PATH
    L = ctypes.CDLL(str(LIB_PATH))
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(xgb_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def _cmp_basis(ob, nb):
    qs, ds, cj, _ = nb.info()
    assert qs == ob.qs and ds == ob.dims and cj == ob.CONJ
    for i, q in enumerate(qs):
        nt, ot = nb.trees(i), ob.trees[q]
        assert len(nt) == len(ot)
        for a, b in zip(nt, ot):
            assert (a[0], a[1], a[2], a[3]) == (b.qu, b.qi, b.qc, b.dims)
            assert a[4] == sum(1 << k for k, d in enumerate(b.dual) if d)


CASES = [
    ("u1", [(2, 2), (0, 1), (-1, 1), (-3, 1)], [(-2, 2), (1, 3)]),
    ("fu1", [(-1, 2), (0, 1), (1, 2), (2, 1)], [(0, 2), (1, 1), (-1, 1)]),
    ("z2", [(0, 2), (1, 3)], [(1, 1), (0, 2)]),
    ("fz2", [(0, 2), (1, 1)], [(1, 2), (0, 1)]),
    ("su2", [(1, 2), (2, 1), (3, 1)], [(1, 1), (2, 2)]),
]


@pytest.mark.parametrize("symname,pB,pC", CASES)
def test_bases_and_trees(symname, pB, pC):
    s, oB, nB = pair_basis(symname, pB)
    _, oC, nC = pair_basis(symname, pC)
    _cmp_basis(oB, nB)
    _cmp_basis(oB.conj(), nB.conj())
    _cmp_basis(oB.combine(oC), nB.combine(nC))
    _cmp_basis(oB.combine(oC).combine(oB.conj()), nB.combine(nC).combine(nB.conj()))
    _cmp_basis(oB.combine(oC).forget_history(), nB.combine(nC).forget_history())


def emulate_permute(tasks, contribs, src, n_out):
    dst = np.zeros(n_out)
    for t in tasks:
        dims = list(t.dims[:t.rank])
        for e in range(t.nelem):
            rem, idx = e, []
            for d in dims:
                idx.append(rem % d)
                rem //= d
            do = t.dst_base + sum(i * s for i, s in zip(idx, t.dst_stride[:t.rank]))
            v = 0.0
            for c in contribs[t.contrib0:t.contrib0 + t.n_contrib]:
                v += c.coeff * src[c.src_base + sum(i * s for i, s in zip(idx, c.src_stride[:t.rank]))]
            dst[do] = v
    return dst


@pytest.mark.parametrize("symname,pB,pC", CASES)
def test_permute_plans_match_oracle(symname, pB, pC):
    from xped_gb300 import Tensor
    rng = np.random.default_rng(0)
    s, oB, nB = pair_basis(symname, pB)
    _, oC, nC = pair_basis(symname, pC)
    ot = oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)
    nt = Tensor.meta([nB, nC], [nB, nC])
    assert nt.sectors()[0] == ot.sectors
    src = ot.data()
    tol = 1e-13 if symname == "su2" else 0.0
    for p in itertools.permutations(range(4)):
        for shift in range(-2, 3):
            ref = ot.permute(shift, list(p))
            tasks, contribs, outm = nt.permute_plan(shift, list(p))
            qs, rows, cols = outm.sectors()
            assert qs == ref.sectors
            assert rows == [b.shape[0] for b in ref.blocks] and cols == [b.shape[1] for b in ref.blocks]
            got = emulate_permute(tasks, contribs, src, outm.size)
            assert np.abs(got - ref.data()).max() <= tol


def test_twist_folded_into_permute_plan():
    from xped_gb300 import Tensor
    rng = np.random.default_rng(1)
    s, oB, nB = pair_basis("fu1", CASES[1][1])
    _, oC, nC = pair_basis("fu1", CASES[1][2])
    ot = oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)
    nt = Tensor.meta([nB, nC], [nB, nC])
    for mask in range(16):
        o2 = ot
        for l in range(4):
            if mask >> l & 1:
                o2 = o2.twist(l)
        for p, shift in [((0, 1, 2, 3), 0), ((0, 2, 1, 3), 0), ((3, 1, 0, 2), 1)]:
            tasks, contribs, outm = nt.permute_plan(shift, list(p), mask)
            got = emulate_permute(tasks, contribs, ot.data(), outm.size)
            assert np.array_equal(got, o2.permute(shift, list(p)).data())


def test_gemm_plan_matches_oracle():
    from xped_gb300 import Tensor
    rng = np.random.default_rng(3)
    s, oB, nB = pair_basis("u1", [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)])
    _, oC, nC = pair_basis("u1", [(-1, 3), (0, 5), (1, 2), (3, 1)])
    o1 = oracle.Tensor(s, [oB, oB], [oC, oB]).set_random(rng)
    o2 = oracle.Tensor(s, [oC, oB], [oB, oC]).set_random(rng)
    n1 = Tensor.meta([nB, nB], [nC, nB])
    n2 = Tensor.meta([nC, nB], [nB, nC])
    descs, out = n1.gemm_plan(n2)
    ref = o1 * o2
    assert out.sectors()[0] == ref.sectors
    # execute the descriptors with numpy
    A, B = o1.data(), o2.data()
    C = np.full(out.size, np.nan)
    for d in descs:
        a = A[d.a_off:d.a_off + d.lda * d.k].reshape((d.lda, d.k), order="F")[:d.m] if d.k else np.zeros((d.m, 0))
        b = B[d.b_off:d.b_off + d.ldb * d.n].reshape((d.ldb, d.n), order="F")[:d.k] if d.k else np.zeros((0, d.n))
        C[d.c_off:d.c_off + d.m * d.n] = (a @ b).ravel(order="F")
    assert np.allclose(C, ref.data(), rtol=1e-13, atol=1e-13)
    flops = sum(2 * d.m * d.n * d.k for d in descs)
    assert flops == sum(2 * a.shape[0] * a.shape[1] * o2.block(q).shape[1]
                        for q, a in zip(o1.sectors, o1.blocks) if o2.has(q))


def test_contract_permutations_match_oracle():
    from xped_gb300 import contract_perms
    cases = [([1, 2, -1, -2, 3], 2, [1, 2, 3, -3, -4], 3, 2), ([-1, 1, -2, -3, 2], 2, [-4, 1, 2, -5, -6], 3, 3),
             ([1, -1, -2, 2, -3, -4], 3, [-5, 1, 2], 1, 4), ([-1, 1], 0, [1, -2, -3, -4], 1, 1),
             ([-1, 2, -4, 1, -5, -2, 3], 3, [1, -6, 3, -3, 2], 2, 3), ([-2, -3, -4, 1, 2, 3], 3, [1, 2, 3, -1], 3, 1)]
    for a1, r1, a2, r2, rr in cases:
        assert list(contract_perms(a1, r1, a2, r2, rr)) == list(get_permutations(a1, r1, a2, r2, rr))


def test_ctm_shapes_metadata_only():
    """Sector structure of the U(1) D=4 chi=32 CTM after init (no GPU): corner
    and edge tensors built by the oracle have the ranks the reference gives."""
    from oracle.basis import Qbasis
    from oracle.ctm import CTM, IPEPS
    s = oracle.U1()
    aux = Qbasis.from_pairs(s, [(-1, 1), (0, 2), (1, 1)])
    phys = Qbasis.from_pairs(s, [(-1, 1), (1, 1)])
    c = CTM(IPEPS(s, aux, phys).set_random(np.random.default_rng(0)), 8).init()
    assert (c.C1.rank, c.C1.corank) == (0, 2) and (c.C2.rank, c.C2.corank) == (1, 1)
    assert (c.C3.rank, c.C3.corank) == (2, 0) and (c.C4.rank, c.C4.corank) == (1, 1)
    assert (c.T1.rank, c.T1.corank) == (1, 3) and (c.T2.rank, c.T2.corank) == (3, 1)
    assert (c.T3.rank, c.T3.corank) == (3, 1) and (c.T4.rank, c.T4.corank) == (1, 3)
