"""CPU-side checks of the native library: it loads, exports every symbol the
headers declare, and its host metadata (bases, fusion trees, sector order,
permute and GEMM plans) matches the oracle bit for bit.  The permute plans
are executed here by numpy emulations of the index arithmetic of both permute
kernels (the row cursor and the wide-row form)."""
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


def emulate_permute(tasks, contribs, src, n_out, sms=152):
    """The index arithmetic of permute_rows_kernel: rows along output leg 0 (row_start prefix
    sums, group size G from the element-weighted row length as perm_rows computes it), the
    launch grid of launch_permute, chunks of 8 consecutive rows per group (the first row decoded,
    the next ones stepped like an odometer, leg 1 fastest) and lane l taking row elements l, l + G,
    ...; every source and destination index is checked against its buffer and every output
    element is written at most once."""
    n = len(tasks)
    row_start = [0]
    elems = weighted = 0.0
    for t in tasks:
        d0 = max(t.dims[0], 1) if t.rank > 0 else 1
        row_start.append(row_start[-1] + t.nelem // d0)
        elems += t.nelem
        weighted += t.nelem * d0
    total_rows = row_start[-1]
    avg = weighted / elems if elems > 0 else 1.0
    G = 1
    while G < 32 and 2.0 * G <= avg * 1.25:
        G *= 2
    dst = np.zeros(n_out)
    if total_rows == 0:
        return dst
    RPC = 8
    per_block = 256 // G
    blocks = max(1, min(sms * 16, ((total_rows + RPC - 1) // RPC + per_block - 1) // per_block))
    ngroups = blocks * 256 // G
    nchunks = (total_rows + RPC - 1) // RPC
    seen = np.zeros(n_out, dtype=np.int64)

    def seek(r):
        ti = int(np.searchsorted(row_start, r, side="right") - 1)
        assert 0 <= ti < n and row_start[ti] <= r < row_start[ti + 1]
        t = tasks[ti]
        rem = r - row_start[ti]
        idx = [0] * 8
        dofs = t.dst_base
        single = t.n_contrib == 1
        sofs = contribs[t.contrib0].src_base if single else 0
        for k in range(1, t.rank):
            idx[k] = rem % t.dims[k]
            rem //= t.dims[k]
            dofs += idx[k] * t.dst_stride[k]
            if single:
                sofs += idx[k] * contribs[t.contrib0].src_stride[k]
        return {"ti": ti, "end": row_start[ti + 1], "idx": idx, "dofs": dofs, "sofs": sofs}

    def step(c, t, cc):
        for k in range(1, t.rank):
            c["dofs"] += t.dst_stride[k]
            if cc is not None:
                c["sofs"] += cc.src_stride[k]
            c["idx"][k] += 1
            if c["idx"][k] < t.dims[k]:
                return
            c["idx"][k] = 0
            c["dofs"] -= t.dims[k] * t.dst_stride[k]
            if cc is not None:
                c["sofs"] -= t.dims[k] * cc.src_stride[k]

    for chunk in range(nchunks):
        assert chunk % ngroups < ngroups  # owned by group chunk mod ngroups
        r0, r1 = chunk * RPC, min(chunk * RPC + RPC, total_rows)
        cur = seek(r0)
        for r in range(r0, r1):
            if r >= cur["end"]:
                cur = seek(r)
            t = tasks[cur["ti"]]
            d0 = t.dims[0] if t.rank > 0 else 1
            ds0 = t.dst_stride[0] if t.rank > 0 else 0
            single = t.n_contrib == 1
            for lane in range(G):
                for i in range(lane, d0, G):
                    if single:
                        cc = contribs[t.contrib0]
                        so = cur["sofs"] + i * (cc.src_stride[0] if t.rank > 0 else 0)
                        assert 0 <= so < len(src)
                        v = cc.coeff * src[so]
                    else:
                        v = 0.0
                        for cc in contribs[t.contrib0:t.contrib0 + t.n_contrib]:
                            so = cc.src_base + i * (cc.src_stride[0] if t.rank > 0 else 0)
                            so += sum(cur["idx"][k] * cc.src_stride[k] for k in range(1, t.rank))
                            assert 0 <= so < len(src)
                            v += cc.coeff * src[so]
                    do = cur["dofs"] + i * ds0
                    assert 0 <= do < n_out
                    dst[do] = v
                    seen[do] += 1
            step(cur, t, contribs[t.contrib0] if single else None)
    assert seen.max() <= 1  # tasks tile disjoint regions of the output
    return dst


def _perm_rows(tasks):
    row_start = [0]
    elems = weighted = 0.0
    for t in tasks:
        d0 = max(t.dims[0], 1) if t.rank > 0 else 1
        row_start.append(row_start[-1] + t.nelem // d0)
        elems += t.nelem
        weighted += t.nelem * d0
    avg = weighted / elems if elems > 0 else 1.0
    G = 1
    while G < 32 and 2.0 * G <= avg * 1.25:
        G *= 2
    return row_start, G


def emulate_permute_wide(tasks, contribs, src, n_out, sms=152):
    """The index arithmetic of permute_rows_wide_kernel: 128-thread CTAs (at most six per SM),
    chunks of 8 rows taken per warp (chunk = warp * (32 / G) + group, stepping by all warps'
    groups), decoder lane u of a group decoding row 8 * chunk + u from scratch (task by search,
    multi-index by division), lane gl copying elements j * G + gl (j = 0, 1) of every row of the
    chunk and the rest of a long row from 2G + gl on in steps of G.  Every chunk must be visited
    once, every index must lie inside its buffer and every output element is written at most once."""
    n = len(tasks)
    row_start, G = _perm_rows(tasks)
    assert G >= 8 and all(t.n_contrib == 1 for t in tasks)
    total_rows = row_start[-1]
    dst = np.zeros(n_out)
    if total_rows == 0:
        return dst
    RPC, SLOTS, THREADS = 8, 2, 128
    gpw = 32 // G
    nchunks = (total_rows + RPC - 1) // RPC
    per_block = THREADS // G
    blocks = max(1, min(sms * 6, (nchunks + per_block - 1) // per_block))
    nwarps = blocks * THREADS // 32
    step = nwarps * gpw
    seen = np.zeros(n_out, dtype=np.int64)
    visited = np.zeros(nchunks, dtype=np.int64)

    def decode(r):
        ti = int(np.searchsorted(row_start, r, side="right") - 1)
        assert 0 <= ti < n and row_start[ti] <= r < row_start[ti + 1]
        t, c = tasks[ti], contribs[tasks[ti].contrib0]
        rem = r - row_start[ti]
        dofs, sofs = t.dst_base, c.src_base
        for k in range(1, t.rank):
            ik = rem % t.dims[k]
            rem //= t.dims[k]
            dofs += ik * t.dst_stride[k]
            sofs += ik * c.src_stride[k]
        ln = t.dims[0] if t.rank > 0 else 1
        ds0 = t.dst_stride[0] if t.rank > 0 else 0
        ss0 = c.src_stride[0] if t.rank > 0 else 0
        return dofs, sofs, ln, ds0, ss0, c.coeff

    for warp in range(nwarps):
        cb = warp * gpw
        while cb < nchunks:
            for g in range(gpw):
                chunk = cb + g
                if chunk >= nchunks:
                    continue
                visited[chunk] += 1
                for u in range(RPC):
                    r = chunk * RPC + u
                    if r >= total_rows:
                        continue
                    dofs, sofs, ln, ds0, ss0, coeff = decode(r)
                    head = [j * G + gl for j in range(SLOTS) for gl in range(G)]
                    tail = [i for gl in range(G) for i in range(SLOTS * G + gl, ln, G)]
                    i = np.array([x for x in head if x < ln] + tail, dtype=np.int64)
                    assert sorted(i.tolist()) == list(range(ln))
                    so, do = sofs + i * ss0, dofs + i * ds0
                    assert so.min() >= 0 and so.max() < len(src) and do.min() >= 0 and do.max() < n_out
                    dst[do] = coeff * src[so]
                    np.add.at(seen, do, 1)
            cb += step
    assert (visited == 1).all()
    assert seen.max() <= 1
    return dst


def run_permute_plan(tasks, contribs, src, n_out):
    """The kernel launch_permute picks: the wide-row kernel for single-contribution plans whose
    groups have 8 or more lanes, the cursor kernel otherwise."""
    _, G = _perm_rows(tasks)
    if G >= 8 and all(t.n_contrib == 1 for t in tasks):
        return emulate_permute_wide(tasks, contribs, src, n_out)
    return emulate_permute(tasks, contribs, src, n_out)


# degeneracies large enough that most permute plans take the wide-row kernel
WIDE_CASES = [
    ("u1", [(-1, 2), (0, 10), (1, 3)], [(0, 4), (1, 13), (2, 1)]),
    ("fz2", [(0, 9), (1, 14)], [(0, 2), (1, 11)]),
]


@pytest.mark.parametrize("symname,pB,pC", WIDE_CASES)
def test_wide_permute_plans_match_oracle(symname, pB, pC):
    from xped_gb300 import Tensor
    rng = np.random.default_rng(4)
    s, oB, nB = pair_basis(symname, pB)
    _, oC, nC = pair_basis(symname, pC)
    ot = oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)
    nt = Tensor.meta([nB, nC], [nB, nC])
    src = ot.data()
    wide = 0
    for p, shift in [((0, 1, 2, 3), 0), ((0, 2, 1, 3), 0), ((1, 0, 3, 2), 1), ((3, 1, 0, 2), -1), ((2, 3, 0, 1), 2),
                     ((1, 3, 2, 0), -2)]:
        ref = ot.permute(shift, list(p))
        tasks, contribs, outm = nt.permute_plan(shift, list(p))
        wide += _perm_rows(tasks)[1] >= 8
        got = run_permute_plan(tasks, contribs, src, outm.size)
        assert np.array_equal(got, ref.data())
    assert wide >= 3


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
