"""Device results against the committed golden fixtures (oracle outputs on seeded
inputs, tests/golden/oracle_golden.npz), through the C-ABI. Tolerances as in the
live-oracle parity tests: FP64 GEMM and permute data 1e-12 relative to the block
scale, singular values, truncation weight and entropy 1e-10; permutes of abelian
tensors bit-exact, SU(2) 1e-13."""
import os

import numpy as np
import pytest

import golden_cases as gc
from helpers import pair_basis, to_native

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    with np.load(os.path.join(HERE, gc.GOLDEN)) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("seed", gc.CHAIN_SEEDS)
def test_chain_matches_golden(gold, seed):
    o1, o2 = gc.chain_inputs(seed)
    _, _, nB = pair_basis("u1", gc.CHAIN_PAIRS, sort=True)
    n1 = to_native(o1, [nB, nB], [nB, nB])
    n2 = to_native(o2, [nB, nB], [nB, nB])
    prod = n1 * n2
    perm = prod.permute(0, [0, 2, 1, 3])
    _, S, _, tw, ent, _ = perm.tSVD(16, 1e-10)
    qs, rs, _ = S.sectors()
    rec = gc.chain_record(prod.data(), perm.data(), list(qs), list(rs), S.data(), tw, ent)
    gc.compare_chain(gold, f"chain_{seed}", rec, 1e-12, 1e-10)


@pytest.mark.parametrize("symname,pB,pD", gc.SYM_CHAINS)
def test_sym_chain_matches_golden(gold, symname, pB, pD):
    oL, oR = gc.sym_chain_inputs(symname, pB, pD)
    _, _, nB = pair_basis(symname, pB)
    _, _, nD = pair_basis(symname, pD)
    nL = to_native(oL, [nB, nB], [nD])
    nR = to_native(oR, [nD], [nB, nB])
    prod = nL * nR
    perm = prod.permute(0, [0, 2, 1, 3])
    _, S, _, tw, ent, _ = perm.tSVD(12, 1e-10)
    qs, rs, _ = S.sectors()
    rec = gc.chain_record(prod.data(), perm.data(), list(qs), list(rs), S.data(), tw, ent)
    gc.compare_chain(gold, f"symchain_{symname}", rec, 1e-12, 1e-10)


@pytest.mark.parametrize("symname,pB,pC", gc.PERMUTE_CASES)
def test_permutes_match_golden(gold, symname, pB, pC):
    ot = gc.permute_input(symname, pB, pC)
    _, _, nB = pair_basis(symname, pB)
    _, _, nC = pair_basis(symname, pC)
    nt = to_native(ot, [nB, nC], [nB, nC])
    tol = 1e-13 if symname == "su2" else 0.0
    for i, (shift, p) in enumerate(gc.PERMUTES):
        r = nt.permute(shift, list(p))
        key = gc.permute_key(symname, i)
        assert list(r.sectors()[0]) == gold[f"{key}_sectors"].tolist()
        gc.compare_digest(gold, key, r.data(), tol, tol)
