"""Seeded cases behind the committed golden fixtures (tests/golden/oracle_golden.npz).

The reference ships no golden vectors: its tests draw bases and entries from
std::random_device and check identities only. These fixtures hold oracle outputs
on seeded inputs instead. tests/golden/make_golden.py writes them; the CPU suite
checks that the oracle still reproduces them; the GPU suite checks the device
results against the same numbers.

Every case is a function of a seed. Large outputs are stored as a strided sample
plus their sum and sum of squares.
"""
from __future__ import annotations

import numpy as np

import oracle
from oracle.basis import Qbasis

GOLDEN = "golden/oracle_golden.npz"
STRIDE = 97
FULL_LIMIT = 4096  # outputs up to this many elements are stored whole

# Tensor<2,2> op chain (every leg q = -2..2, deg [2, 4, 6, 4, 2]): T1*T2 -> permute<0>(0,2,1,3) -> tSVD(16, 1e-10)
CHAIN_PAIRS = [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)]
CHAIN_SEEDS = (0, 1, 2)

# permutes of rank-(2,2) tensors with legs [B, C | B, C]
PERMUTE_CASES = [
    ("u1", [(2, 2), (0, 1), (-1, 1), (-3, 1)], [(-2, 2), (1, 3)]),
    ("fu1", [(-1, 2), (0, 1), (1, 2), (2, 1)], [(0, 2), (1, 1), (-1, 1)]),
    ("fz2", [(0, 2), (1, 3)], [(1, 2), (0, 1)]),
    ("su2", [(1, 2), (2, 1), (3, 1)], [(1, 1), (2, 2)]),
]
PERMUTES = [(1, (2, 0, 3, 1)), (-1, (1, 3, 0, 2)), (0, (3, 2, 1, 0))]


def chain_inputs(seed):
    rng = np.random.default_rng(seed)
    s = oracle.make_symmetry("u1")
    B = Qbasis.from_pairs(s, CHAIN_PAIRS, sort=True)
    o1 = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    o2 = oracle.Tensor(s, [B, B], [B, B]).set_random(rng)
    return o1, o2


def permute_input(symname, pB, pC, seed=0):
    rng = np.random.default_rng(seed)
    s = oracle.make_symmetry(symname)
    oB, oC = Qbasis.from_pairs(s, pB), Qbasis.from_pairs(s, pC)
    return oracle.Tensor(s, [oB, oC], [oB, oC]).set_random(rng)


def digest(x):
    """Whole array when small, else a strided sample with sum and sum of squares."""
    x = np.asarray(x, dtype=np.float64).ravel()
    if x.size <= FULL_LIMIT:
        return {"full": x}
    return {"sample": x[::STRIDE].copy(), "sum": np.array([x.sum()]), "sumsq": np.array([np.dot(x, x)])}


def sigma_blocks(sectors, rows, data):
    """Diagonals of the k x k column-major S blocks, sector by sector."""
    out, off = [], 0
    for k in rows:
        out.append(np.asarray(data[off:off + k * k]).reshape((k, k), order="F").diagonal().copy())
        off += k * k
    return np.concatenate(out) if out else np.zeros(0)


def chain_record(prod_data, perm_data, s_sectors, s_rows, s_data, tw, ent):
    rec = {}
    for name, arr in (("prod", prod_data), ("perm", perm_data)):
        for k, v in digest(arr).items():
            rec[f"{name}_{k}"] = v
    rec["sigma"] = sigma_blocks(s_sectors, s_rows, s_data)
    rec["s_sectors"] = np.asarray(s_sectors, dtype=np.int64)
    rec["s_rows"] = np.asarray(s_rows, dtype=np.int64)
    rec["tw_ent"] = np.array([tw, ent])
    return rec


def oracle_chain(seed):
    o1, o2 = chain_inputs(seed)
    prod = o1 * o2
    perm = prod.permute(0, [0, 2, 1, 3])
    _, S, _, tw, ent = perm.tsvd(16, 1e-10)
    return chain_record(prod.data(), perm.data(), S.sectors, [b.shape[0] for b in S.blocks], S.data(), tw, ent)


# fermionic Z2 and SU(2) op chains: L [B, B | D] * R [D | B, B] -> permute<0>(0,2,1,3) -> tSVD(12, 1e-10)
SYM_CHAINS = [
    ("fz2", [(0, 2), (1, 3)], [(0, 3), (1, 2)]),
    ("su2", [(1, 2), (2, 1), (3, 1)], [(1, 2), (2, 2), (3, 1)]),
]
SYM_CHAIN_SEED = 3


def sym_chain_inputs(symname, pB, pD):
    rng = np.random.default_rng(SYM_CHAIN_SEED)
    s = oracle.make_symmetry(symname)
    B, D = Qbasis.from_pairs(s, pB), Qbasis.from_pairs(s, pD)
    oL = oracle.Tensor(s, [B, B], [D]).set_random(rng)
    oR = oracle.Tensor(s, [D], [B, B]).set_random(rng)
    return oL, oR


def oracle_sym_chain(symname, pB, pD):
    oL, oR = sym_chain_inputs(symname, pB, pD)
    prod = oL * oR
    perm = prod.permute(0, [0, 2, 1, 3])
    _, S, _, tw, ent = perm.tsvd(12, 1e-10)
    return chain_record(prod.data(), perm.data(), S.sectors, [b.shape[0] for b in S.blocks], S.data(), tw, ent)


def permute_key(symname, i):
    return f"permute_{symname}_{i}"


def oracle_permutes():
    out = {}
    for symname, pB, pC in PERMUTE_CASES:
        t = permute_input(symname, pB, pC)
        for i, (shift, p) in enumerate(PERMUTES):
            r = t.permute(shift, list(p))
            for k, v in digest(r.data()).items():
                out[f"{permute_key(symname, i)}_{k}"] = v
            out[f"{permute_key(symname, i)}_sectors"] = np.asarray(r.sectors, dtype=np.int64)
    return out


def compare_digest(gold, prefix, x, rtol, atol=0.0):
    """Compare array x with the stored digest under `prefix`; returns the largest error."""
    x = np.asarray(x, dtype=np.float64).ravel()
    if f"{prefix}_full" in gold:
        ref = gold[f"{prefix}_full"]
        assert x.shape == ref.shape, (prefix, x.shape, ref.shape)
        scale = max(1.0, float(np.abs(ref).max()) if ref.size else 1.0)
        err = float(np.abs(x - ref).max()) if ref.size else 0.0
        assert err <= atol + rtol * scale, (prefix, err)
        return err
    ref = gold[f"{prefix}_sample"]
    got = x[::STRIDE]
    assert got.shape == ref.shape, (prefix, got.shape, ref.shape)
    scale = max(1.0, float(np.abs(ref).max()))
    err = float(np.abs(got - ref).max())
    assert err <= atol + rtol * scale, (prefix, err)
    s, ss = float(gold[f"{prefix}_sum"][0]), float(gold[f"{prefix}_sumsq"][0])
    assert abs(x.sum() - s) <= atol + rtol * max(1.0, np.sqrt(ss)) * np.sqrt(x.size), (prefix, "sum")
    assert abs(np.dot(x, x) - ss) <= atol + rtol * max(1.0, ss), (prefix, "sumsq")
    return err


def compare_chain(gold, p, rec, rtol_data, rtol_sigma):
    """Compare a chain record with the fixture arrays stored under prefix `p`."""
    assert np.array_equal(rec["s_sectors"], gold[f"{p}_s_sectors"])
    assert np.array_equal(rec["s_rows"], gold[f"{p}_s_rows"])
    for name in ("prod", "perm"):
        key = "full" if f"{name}_full" in rec else "sample"
        if key == "full":
            compare_digest(gold, f"{p}_{name}", rec[f"{name}_full"], rtol_data)
        else:
            ref = gold[f"{p}_{name}_sample"]
            scale = max(1.0, float(np.abs(ref).max()))
            assert np.abs(rec[f"{name}_sample"] - ref).max() <= rtol_data * scale, (p, name)
            ss = float(gold[f"{p}_{name}_sumsq"][0])
            assert abs(float(rec[f"{name}_sumsq"][0]) - ss) <= rtol_data * max(1.0, ss), (p, name, "sumsq")
    sig, ref = rec["sigma"], gold[f"{p}_sigma"]
    assert sig.shape == ref.shape
    assert np.abs(sig - ref).max() <= rtol_sigma * max(1.0, float(ref.max()))
    tw, ent = rec["tw_ent"]
    gtw, gent = gold[f"{p}_tw_ent"]
    assert abs(tw - gtw) <= rtol_sigma * max(1.0, abs(gtw))
    assert abs(ent - gent) <= rtol_sigma * max(1.0, abs(gent))
