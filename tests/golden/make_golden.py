"""Writes tests/golden/oracle_golden.npz: oracle outputs on the seeded cases of
tests/golden_cases.py (U(1) Tensor<2,2> op chains, fermionic Z2 and SU(2) op
chains, permutes of U(1), fermionic U(1), fermionic Z2 and SU(2) tensors).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import golden_cases as gc  # noqa: E402


def main():
    out = {}
    for seed in gc.CHAIN_SEEDS:
        for k, v in gc.oracle_chain(seed).items():
            out[f"chain_{seed}_{k}"] = v
    for symname, pB, pD in gc.SYM_CHAINS:
        for k, v in gc.oracle_sym_chain(symname, pB, pD).items():
            out[f"symchain_{symname}_{k}"] = v
    out.update(gc.oracle_permutes())
    path = os.path.join(HERE, "oracle_golden.npz")
    np.savez_compressed(path, **out)
    print(path, len(out), "arrays", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
