"""The oracle reproduces the committed golden fixtures (tests/golden/oracle_golden.npz,
written by tests/golden/make_golden.py): a change of the oracle's arithmetic or
ordering shows up here before it reaches a parity test."""
import os

import numpy as np
import pytest

import golden_cases as gc

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    with np.load(os.path.join(HERE, gc.GOLDEN)) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("seed", gc.CHAIN_SEEDS)
def test_oracle_chain_matches_golden(gold, seed):
    gc.compare_chain(gold, f"chain_{seed}", gc.oracle_chain(seed), 1e-13, 1e-13)


@pytest.mark.parametrize("symname,pB,pD", gc.SYM_CHAINS)
def test_oracle_sym_chain_matches_golden(gold, symname, pB, pD):
    gc.compare_chain(gold, f"symchain_{symname}", gc.oracle_sym_chain(symname, pB, pD), 1e-13, 1e-13)


def test_oracle_permutes_match_golden(gold):
    for symname, pB, pC in gc.PERMUTE_CASES:
        t = gc.permute_input(symname, pB, pC)
        tol = 1e-14 if symname == "su2" else 0.0
        for i, (shift, p) in enumerate(gc.PERMUTES):
            r = t.permute(shift, list(p))
            key = gc.permute_key(symname, i)
            assert r.sectors == gold[f"{key}_sectors"].tolist()
            gc.compare_digest(gold, key, r.data(), tol, tol)


def test_golden_digest_rejects_a_planted_change(gold):
    """The comparison is not vacuous: one changed element of a stored output fails it."""
    t = gc.permute_input(*gc.PERMUTE_CASES[0])
    x = t.permute(*(lambda s, p: (s, list(p)))(*gc.PERMUTES[0])).data().copy()
    x[len(x) // 2] += 1e-9
    with pytest.raises(AssertionError):
        gc.compare_digest(gold, gc.permute_key(gc.PERMUTE_CASES[0][0], 0), x, 0.0, 0.0)
