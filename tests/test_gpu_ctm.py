"""CTMRG moves on the GPU against the oracle (1x1 cell, U(1) and fermionic Z2).

The SVD gauge is fixed identically on both sides (largest |u_i| positive), so
environments are compared entry by entry; tolerance 1e-10 relative to the
largest entry after several full steps (the FP64 contract tolerance: FP64
round-off accumulates through ~100 contractions and four truncated SVDs per
step)."""
import numpy as np
import pytest

from oracle.basis import Qbasis
from oracle.ctm import CTM as OCTM
from oracle.ctm import IPEPS
import oracle
from helpers import assert_same, pair_basis, to_native

pytestmark = pytest.mark.gpu


def _setup(symname, aux_pairs, phys_pairs, chi, seed):
    from xped_gb300 import CTM
    s, oaux, naux = pair_basis(symname, aux_pairs, sort=True)
    _, ophys, nphys = pair_basis(symname, phys_pairs, sort=True)
    rng = np.random.default_rng(seed)
    peps = IPEPS(s, oaux, ophys).set_random(rng)
    nA = to_native(peps.A, [naux, naux], [naux, naux, nphys])
    return OCTM(peps, chi).init(), CTM(nA, chi).init()


def _compare(oc, nc, rtol):
    env = oc.env()
    for name, t in nc.env().items():
        assert_same(t, env[name], rtol, rtol)


def test_ctm_init_u1():
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 8, 0)
    _compare(oc, nc, 1e-12)
    assert_same(nc.get("Adag"), oc.peps.Adag, 0, 0)


@pytest.mark.parametrize("seed", [0, 1])
def test_ctm_steps_u1_small(seed):
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 12, seed)
    for _ in range(3):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-10)


def test_ctm_u1_d4_chi32_step():
    """U(1) iPEPS CTMRG steps: phys dim 2, D=4 (q -1..1 deg [1,2,1]), chi=32."""
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    for _ in range(2):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-10)


def test_ctm_fermionic_z2():
    oc, nc = _setup("fz2", [(0, 2), (1, 2)], [(0, 1), (1, 1)], 10, 3)
    _compare(oc, nc, 1e-12)
    for _ in range(2):
        oc.grow_all()
        nc.grow_all()
    _compare(oc, nc, 1e-10)


def test_rdm_and_energy_match_oracle():
    """computeRDM_h / computeRDM_v and the Heisenberg bond energies after three steps."""
    from oracle.ctm import bond_expectation as obond
    from oracle.ctm import heisenberg_u1
    from xped_gb300 import bond_expectation
    from xped_gb300.observables import heisenberg_bond
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 12, 0)
    for _ in range(3):
        oc.grow_all()
        nc.grow_all()
    s = oracle.make_symmetry("u1")
    oH = heisenberg_u1(s, oc.peps.A.cod[2])
    nH = heisenberg_bond(nc.get("A").leg(4))
    assert_same(nH, oH, 0, 0)
    for orho, nrho in ((oc.rdm_h(), nc.rdm_h()), (oc.rdm_v(), nc.rdm_v())):
        assert_same(nrho, orho, 1e-10, 1e-10)
        assert abs(bond_expectation(nrho, nH) - obond(orho, oH)) < 1e-10


def test_randomized_projectors_keep_the_energy():
    """Chosen form (randomized projector SVD with history widths: three
    subspace iterations, last kept + max(16, 50 %) columns) against the exact
    FP64 tSVD on the GPU: same kept counts every step and the same energy per
    site to 1e-8."""
    from xped_gb300.observables import energy, heisenberg_bond
    _, ex = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    _, rz = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    rz.set_svd("randomized", power_iters=3, oversample=16, growth=0.5)
    ex.record(True)
    rz.record(True)
    for _ in range(6):
        ex.grow_all()
        rz.grow_all()
    H = heisenberg_bond(ex.get("A").leg(4))
    e_ex, e_rz = energy(ex, H), energy(rz, H)
    assert abs(e_ex - e_rz) < 1e-8, (e_ex, e_rz)
    st = rz.stats()
    assert st["sketched_sectors"] > 0
    for a, b in zip(ex.records(), rz.records()):
        assert a["sectors"] == b["sectors"]
        assert list(a["keep"]) == list(b["keep"])


def test_oracle_copy_of_device_ctm_continues_identically():
    """A device CTM copied into the oracle (same bases, sectors and data)
    gives the same environment after one more step on both sides."""
    from oracle.convert import ctm_from_native
    _, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 12, 2)
    for _ in range(2):
        nc.grow_all()
    s = oracle.make_symmetry("u1")
    oc = ctm_from_native(s, nc, 12)
    _compare(oc, nc, 0)
    oc.grow_all()
    nc.grow_all()
    _compare(oc, nc, 1e-10)


def test_split_precision_contractions_stay_close():
    """3xTF32 block GEMMs in the corner contractions / renormalisation (the
    projector SVD and construction in FP64): energy per site within 1e-6 of
    the all-FP64 run after four steps."""
    from xped_gb300.observables import energy, heisenberg_bond
    _, ex = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    _, tc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    tc.set_gemm("3xtf32")
    for _ in range(4):
        ex.grow_all()
        tc.grow_all()
    H = heisenberg_bond(ex.get("A").leg(4))
    e_ex, e_tc = energy(ex, H), energy(tc, H)
    print("energy fp64", e_ex, "3xtf32", e_tc, "diff", abs(e_ex - e_tc))
    assert abs(e_ex - e_tc) < 1e-6


def test_warm_started_projectors_keep_the_energy():
    """Randomized projector SVD seeded with each direction's previous V^dag
    (two subspace iterations once seeded): energy per site within 1e-8 of
    the exact FP64 tSVD after six steps."""
    from xped_gb300.observables import energy, heisenberg_bond
    _, ex = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    _, rz = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 32, 7)
    rz.set_svd("randomized", power_iters=3, oversample=16, growth=0.5).set_warm_start(2)
    for _ in range(6):
        ex.grow_all()
        rz.grow_all()
    H = heisenberg_bond(ex.get("A").leg(4))
    e_ex, e_rz = energy(ex, H), energy(rz, H)
    print("energy exact", e_ex, "warm", e_rz, "diff", abs(e_ex - e_rz))
    assert abs(e_ex - e_rz) < 1e-8


def test_tensor_core_sketch_iterations_keep_the_energy():
    """Randomized projector SVD with 8 subspace iterations whose first product and
    first six iterations multiply as 3xTF32 tensor-core GEMMs (the last two
    iterations, the projection and the small SVDs in FP64): energy per site within
    1e-8 of the all-FP64 randomized run and of the exact tSVD after four steps."""
    from xped_gb300.observables import energy, heisenberg_bond
    aux = [(-1, 2), (0, 2), (1, 2)]
    _, ex = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 3)
    _, rz = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 3)
    _, tc = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 3)
    for c in (rz, tc):
        c.set_svd("randomized", power_iters=8, oversample=16, growth=0.5)
    tc.set_sketch_precision(2)
    for _ in range(4):
        ex.grow_all()
        rz.grow_all()
        tc.grow_all()
    assert tc.stats()["sketched_sectors"] > 0
    H = heisenberg_bond(ex.get("A").leg(4))
    e_ex, e_rz, e_tc = energy(ex, H), energy(rz, H), energy(tc, H)
    print("energy exact", e_ex, "fp64 sketch", e_rz, "tc sketch", e_tc, "diff", abs(e_rz - e_tc), abs(e_ex - e_tc))
    assert abs(e_rz - e_tc) < 1e-8
    assert abs(e_ex - e_tc) < 1e-8


def test_solver_converges_like_the_oracle():
    """CTMSolver::solve (src/PEPS/CTMSolver.cpp:50-80) on the device and in the oracle from the same
    FROM_A start: the same number of grow_all steps, energies within 1e-10 after every step."""
    from oracle.ctm import heisenberg_u1
    from xped_gb300.observables import heisenberg_bond
    oc, nc = _setup("u1", [(-1, 1), (0, 2), (1, 1)], [(-1, 1), (1, 1)], 16, 4)
    s = oracle.make_symmetry("u1")
    H = heisenberg_bond(nc.get("A").leg(4))
    oH = heisenberg_u1(s, oc.peps.A.cod[2])
    r = nc.solve(H, tol_E=1e-9, max_steps=40)
    o = oc.solve(oH, tol_E=1e-9, max_steps=40)
    print("device", r["steps"], r["E"], "oracle", o["steps"], o["E"])
    assert r["converged"] and o["converged"]
    assert r["steps"] == o["steps"]
    assert np.abs(np.array(r["energies"]) - np.array(o["energies"])).max() < 1e-10


@pytest.mark.parametrize("svd", ["exact", "randomized"])
def test_fp64_accurate_tensor_core_products_match_fp64(svd):
    """Every block GEMM of the CTM step (corner contractions, renormalisation, the projector product
    T1 T2, the projectors and the randomized SVD's sketch products) on the FP64-accurate tensor-core
    form (exact BF16 slices): environments within 1e-10 and energies within 1e-12 of the all-FP64 run
    after four steps."""
    from xped_gb300.observables import energy, heisenberg_bond
    aux = [(-1, 2), (0, 2), (1, 2)]
    _, ex = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 3)
    _, tc = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 3)
    if svd == "randomized":
        for c in (ex, tc):
            c.set_svd("randomized", power_iters=4, oversample=16, growth=0.5)
    tc.set_gemm("f64tc")
    for _ in range(4):
        ex.grow_all()
        tc.grow_all()
    H = heisenberg_bond(ex.get("A").leg(4))
    e_ex, e_tc = energy(ex, H), energy(tc, H)
    env_ex, env_tc = ex.env(), tc.env()
    err = max(float(np.abs(env_tc[k].data() - env_ex[k].data()).max()) for k in env_ex)
    print(svd, "energy fp64", e_ex, "f64tc", e_tc, "diff", abs(e_ex - e_tc), "env diff", err)
    assert abs(e_ex - e_tc) < 1e-12
    assert err < 1e-10


@pytest.mark.parametrize("gemm", ["fp64", "f64tc"])
def test_concurrent_move_pairs_equal_sequential(gemm):
    """grow_all running the left/right and then the top/bottom moves two at a time on two streams
    (the default with randomized projectors) gives the same environments bit for bit, the same
    statistics and the same decomposition log, in the same order, as the four moves one after the
    other."""
    aux = [(-1, 2), (0, 2), (1, 2)]
    _, seq = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 5)
    _, par = _setup("u1", aux, [(-1, 1), (1, 1)], 48, 5)
    for c in (seq, par):
        c.set_svd("randomized", power_iters=3, oversample=16, growth=0.5)
        c.set_gemm(gemm)
        c.record(True)
    seq.set_concurrent(False)
    par.set_concurrent(True)
    for _ in range(4):
        seq.grow_all()
        par.grow_all()
    env_s, env_p = seq.env(), par.env()
    for k in env_s:
        assert np.array_equal(env_s[k].data(), env_p[k].data()), k
    assert seq.stats() == par.stats()
    rs, rp = seq.records(), par.records()
    assert [r["dir"] for r in rs] == [r["dir"] for r in rp] == [0, 1, 2, 3] * 4
    for a, b in zip(rs, rp):
        assert np.array_equal(a["keep"], b["keep"]) and np.array_equal(a["width"], b["width"])
        assert all(np.array_equal(x, y) for x, y in zip(a["spectrum"], b["spectrum"]))
