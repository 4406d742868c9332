"""Randomized blockwise tSVD (the chosen form) on the GPU.

Parity: with the same seed both the device and the numpy restatement draw
the same Gaussian test matrices, so the whole pipeline (sketch, subspace
iterations, projected SVD, sign convention, truncation) is compared
element by element.  Against the exact FP64 tSVD the randomized form must
keep the same sectors and counts, with kept singular values inside the
stated budget."""
import numpy as np
import pytest

import oracle
from oracle.basis import Qbasis
from oracle.rsvd import tsvd_randomized as oracle_rsvd
from xped_gb300.workloads import power_law_sectors

from helpers import assert_same

pytestmark = pytest.mark.gpu


def _pair(secs):
    from xped_gb300 import Basis, Tensor
    s = oracle.make_symmetry("u1")
    pairs = [(q, n) for q, n, *_ in secs]
    oB = Qbasis.from_pairs(s, pairs, sort=True)
    nB = Basis.from_pairs("U1", pairs, sort=True)
    ot = oracle.Tensor(s, [oB], [oB], fill=False)
    blocks = {q: b for q, _n, _a, _c, b in secs}
    nt = Tensor.zeros([nB], [nB])
    qs = nt.sectors()[0]
    for q in qs:
        ot.push_back(q, blocks[q])
    nt.set_data(ot.data())
    return ot, nt


def _keep_counts(S, sectors):
    qs, rs, _ = S.sectors()
    d = dict(zip(qs, rs))
    return [d.get(q, 0) for q in sectors]


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("power_iters", [0, 1, 2])
def test_rsvd_matches_oracle_same_sketch(seed, power_iters):
    secs = power_law_sectors(seed, size=(16, 160))
    ot, nt = _pair(secs)
    chi = 64
    _U, eS, _V, _tw, _ent, keep_ex = nt.tSVD(chi, 1e-10)
    sketch = [k + 8 for k in keep_ex]
    nU, nS, nV, ntw, nent, nkeep, nwidth, nsat = nt.tSVD_randomized(chi, 1e-10, sketch, power_iters, seed=99)
    oU, oS, oV, otw, oent, okeep, owidth, osat = oracle_rsvd(ot, chi, 1e-10, sketch, power_iters, seed=99)
    assert nwidth == owidth
    assert nkeep == okeep
    assert nsat == osat
    assert_same(nS, oS, 1e-10, 1e-12)
    assert_same(nU, oU, 1e-8, 1e-8)
    assert_same(nV, oV, 1e-8, 1e-8)
    assert abs(ntw - otw) <= 1e-10 * max(1.0, otw)


def test_rsvd_resolves_the_exact_truncation():
    """Kept set identical to the exact FP64 tSVD; kept singular values within
    1e-3 of the largest with 16 extra columns and two subspace iterations on
    power-law spectra (exponents 1-3; exponent 1 converges slowest, the
    numpy restatement reaches 4e-4 on these inputs)."""
    for seed in range(3):
        secs = power_law_sectors(seed, size=(16, 512))
        _ot, nt = _pair(secs)
        chi = 128
        eU, eS, eV, etw, _e, keep_ex = nt.tSVD(chi, 1e-10)
        sketch = [k + 16 for k in keep_ex]
        rU, rS, rV, rtw, _r, keep, width, nsat = nt.tSVD_randomized(chi, 1e-10, sketch, 2, seed=5)
        assert keep == keep_ex
        assert nsat == 0
        es, rs = eS.data(), rS.data()
        assert np.abs(rs - es).max() <= 1e-3 * np.abs(es).max()
        # sketched sectors used fewer columns than the full blocks
        qs, rows, cols = nt.sectors()
        assert sum(width) < sum(min(r, c) for r, c in zip(rows, cols))


def test_rsvd_saturated_sector_falls_back_to_exact():
    secs = power_law_sectors(4, size=(40, 120), alphas=(1.0,))
    ot, nt = _pair(secs)
    chi = 200
    eU, eS, eV, etw, _e, keep_ex = nt.tSVD(chi, 1e-10)
    sketch = [max(1, k // 4) for k in keep_ex]  # far too small: every sketched sector saturates
    rU, rS, rV, rtw, _r, keep, width, nsat = nt.tSVD_randomized(chi, 1e-10, sketch, 1, seed=3)
    oU, oS, oV, otw, _o, okeep, owidth, osat = oracle_rsvd(ot, chi, 1e-10, sketch, 1, seed=3)
    assert nsat == osat and nsat > 0
    assert keep == keep_ex == okeep
    assert_same(rS, oS, 1e-10, 1e-12)
    assert np.allclose(rS.data(), eS.data(), rtol=0, atol=1e-10 * np.abs(eS.data()).max())


def test_rsvd_exact_widths_equal_tsvd():
    """sketch <= 0 everywhere: every sector exact, results equal to tSVD."""
    secs = power_law_sectors(6, size=(8, 64))
    _ot, nt = _pair(secs)
    eU, eS, eV, etw, ee, keep_ex = nt.tSVD(32, 1e-10)
    n = len(nt.sectors()[0])
    rU, rS, rV, rtw, re, keep, width, nsat = nt.tSVD_randomized(32, 1e-10, [0] * n, 1, seed=1)
    assert keep == keep_ex and nsat == 0
    assert np.array_equal(rS.data(), eS.data())
    assert np.array_equal(rU.data(), eU.data())
    assert np.array_equal(rV.data(), eV.data())
    assert rtw == etw and re == ee


def test_rsvd_rank_deficient_blocks():
    """Blocks of exact rank 3 sketched with 8 columns: the zero directions
    are truncated by eps and the kept triplets match the exact tSVD."""
    rng = np.random.default_rng(8)
    secs = []
    for a, n in enumerate([30, 50, 40]):
        blk = rng.standard_normal((n, 3)) @ rng.standard_normal((3, n))
        secs.append((a - 1, n, 0.0, 1.0, blk))
    _ot, nt = _pair(secs)
    eU, eS, eV, *_ , keep_ex = nt.tSVD(100, 1e-10)
    rU, rS, rV, rtw, _r, keep, width, nsat = nt.tSVD_randomized(100, 1e-10, [8, 8, 8], 1, seed=2)
    assert keep == keep_ex == [3, 3, 3]
    assert np.allclose(rS.data(), eS.data(), rtol=1e-11, atol=0)
    assert np.allclose(rU.data(), eU.data(), rtol=0, atol=1e-9)
    assert np.allclose(rV.data(), eV.data(), rtol=0, atol=1e-9)


def test_rsvd_warm_start_matches_oracle():
    """Sketch seeded with the V^dag of a nearby matrix: device and oracle agree
    element by element, and one subspace iteration resolves the truncation
    of the perturbed matrix."""
    from oracle.convert import tensor_from_native
    secs = power_law_sectors(9, size=(24, 160), alphas=(2.0, 3.0))
    ot, nt = _pair(secs)
    rng = np.random.default_rng(10)
    # perturbed copy (same structure)
    pert = [(q, n, a, c, b + 1e-4 * rng.standard_normal(b.shape)) for q, n, a, c, b in secs]
    ot2, nt2 = _pair(pert)
    chi = 48
    _U, _S, nV, *_ = nt.tSVD(chi, 1e-10)
    s = oracle.make_symmetry("u1")
    oV = tensor_from_native(s, nV)
    _U2, eS, _V2, _tw, _e, keep_ex = nt2.tSVD(chi, 1e-10)
    sketch = [k + 8 for k in keep_ex]
    rU, rS, rV, rtw, _r, keep, width, nsat = nt2.tSVD_randomized(chi, 1e-10, sketch, 1, seed=4, warm=nV)
    oU, oS, oVd, otw, _o, okeep, owidth, osat = oracle_rsvd(ot2, chi, 1e-10, sketch, 1, seed=4, warm=oV)
    assert keep == okeep == keep_ex and nsat == osat == 0
    assert_same(rS, oS, 1e-10, 1e-12)
    assert_same(rU, oU, 1e-8, 1e-8)
    assert_same(rV, oVd, 1e-8, 1e-8)
    assert np.abs(rS.data() - eS.data()).max() <= 1e-8 * np.abs(eS.data()).max()
